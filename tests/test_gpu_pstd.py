"""PSTD field step and wire coupling on the GPU vs the oracle (through the C ABI)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import pstd_oracle as PO  # noqa: E402
from oracle import sbe_oracle as O  # noqa: E402

EPSR = 12.9


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


def dev(x):
    return torch.as_tensor(np.ascontiguousarray(x)).cuda().contiguous()


def host(t):
    return t.detach().cpu().numpy()


def smooth_fields(rng, x, ncomp, amp=1.0):
    L = x[-1] - x[0]
    out = np.zeros((ncomp, len(x)), complex)
    for c in range(ncomp):
        for m in range(1, 12):
            a, b = rng.standard_normal(2)
            out[c] += amp * (a + 1j * b) * np.exp(2j * np.pi * m * x / L) / m
    return out


@pytest.mark.parametrize("nx", [256, 1024, 16384, 65536])
def test_grid_and_derivative(nx):
    from pulsesuite_gb300.pstd import Pstd1D
    dx = 10e-9
    p = Pstd1D(nx, dx, EPSR)
    x, q = PO.pstd_grid(nx, dx)
    assert np.array_equal(host(p.x), x)
    assert np.array_equal(host(p.q), q)
    rng = np.random.default_rng(nx)
    f = rng.standard_normal((2, nx)) + 1j * rng.standard_normal((2, nx))
    d2 = host(p.deriv(dev(f)))
    d1 = host(p.deriv(dev(f[1])))
    for c in range(2):
        assert rel(d2[c], PO.deriv(f[c], q)) < 1e-13
    assert rel(d1, PO.deriv(f[1], q)) < 1e-13
    p.close()


def test_steps_with_current_and_absorber_vs_oracle():
    from pulsesuite_gb300.pstd import Pstd1D
    nx, dx, dt = 1024, 10e-9, 0.05e-15
    p = Pstd1D(nx, dx, EPSR, n_abc=64, abc_strength=0.05)
    o = PO.Pstd1D(nx, dx, EPSR, n_abc=64, strength=0.05)
    rng = np.random.default_rng(1)
    E = smooth_fields(rng, o.x, 2, 1e6)
    H = smooth_fields(rng, o.x, 2, 1e3)
    Eg, Hg = dev(E), dev(H)
    for n in range(20):
        J = smooth_fields(rng, o.x, 2, 1e10)
        p.step(Eg, Hg, dev(J), dt)
        E, H = o.step(E, H, J, dt)
    assert rel(host(Eg), E) < 1e-12
    assert rel(host(Hg), H) < 1e-12
    p.close()


def test_energy_invariant_on_gpu():
    from pulsesuite_gb300.pstd import Pstd1D
    nx, dx = 4096, 10e-9
    p = Pstd1D(nx, dx, EPSR)
    o = PO.Pstd1D(nx, dx, EPSR)
    dt = 0.95 * p.max_dt()
    rng = np.random.default_rng(2)
    Eg = dev(smooth_fields(rng, o.x, 2, 1.0))
    Hg = dev(np.zeros((2, nx), complex))
    Hprev = host(Hg)
    p.update_h(Eg, Hg, dt)
    w0 = o.energy(host(Eg), Hprev, host(Hg))
    for n in range(200):
        Hprev = host(Hg)
        p.update_e(Eg, Hg, None, dt)
        p.update_h(Eg, Hg, dt)
        if n % 20 == 19:
            w = o.energy(host(Eg), Hprev, host(Hg))
            assert abs(w - w0) < 1e-11 * w0
    p.close()


def test_unstable_step_is_rejected():
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.pstd import Pstd1D
    p = Pstd1D(256, 10e-9, 1.0)
    E = p.zeros()
    H = p.zeros()
    with pytest.raises(_lib.SbeError, match="unstable"):
        p.step(E, H, None, 1.01 * p.max_dt())
    p.close()


def test_longitudinal_field_vs_oracle():
    from pulsesuite_gb300.pstd import Pstd1D
    nx, dx = 2048, 10e-9
    p = Pstd1D(nx, dx, EPSR)
    x, q = PO.pstd_grid(nx, dx)
    rng = np.random.default_rng(4)
    rho = rng.standard_normal(nx) + 1j * rng.standard_normal(nx)
    px = 1e-9 * (rng.standard_normal(nx) + 1j * rng.standard_normal(nx))
    ex = host(p.elong(dev(rho), dev(px)))
    assert rel(ex, PO.elong(rho, px, q, EPSR)) < 1e-13
    p.close()


MAT = dict(me=0.067 * O.ME0, mh=0.45 * O.ME0, gap=1.52 * O.E0, HO=100e-3 * O.E0, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=EPSR, Oph=36e-3 * O.E0 / O.HBAR,
           Gph=3e-3 * O.E0 / O.HBAR)
ALL = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
           LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)


def _wires(nks):
    from pulsesuite_gb300.wires import WireContext, WireSpec
    Ls = [np.pi / (3e9 / (nk / 2 - 0.5)) for nk in nks]
    specs = [WireSpec(nk=nk, L=L, wire_index=w + 1, flags=dict(ALL), **MAT)
             for w, (nk, L) in enumerate(zip(nks, Ls))]
    return WireContext(specs), [O.Wire(nk, L, MAT, ALL) for nk, L in zip(nks, Ls)]


def test_sample_and_deposit_vs_oracle():
    from pulsesuite_gb300.pstd import CoupledLine, Pstd1D
    nx, dx = 512, 2e-9
    ctx, ows = _wires([16, 32, 24])
    p = Pstd1D(nx, dx, EPSR)
    o = PO.Pstd1D(nx, dx, EPSR)
    wx = [-120e-9, 3.3e-9, 25e-9]
    line = CoupledLine(ctx, p, wx)
    ol = PO.CoupledLine(o, ows, [1, 2, 3], wx)
    rng = np.random.default_rng(6)
    E = smooth_fields(rng, o.x, 2, 1e7)
    Ex = smooth_fields(rng, o.x, 1, 1e5)[0]
    line.sample(dev(Ex), dev(E))
    Ek = host(line.view("Ek"))
    ref = ol.sample(Ex, E)
    for w in range(3):
        got = host(ctx.rvec(line.view("Ek"), w, 3))
        for f in range(3):
            assert rel(got[f], ref[w][f]) < 1e-12, (w, f)
    assert np.isfinite(Ek).all()
    srcs = []
    flat = []
    for w, wi in enumerate(ows):
        r = wi.g["r"]
        s = np.stack([(1.0 + 0.3j * c) * np.cos(np.pi * r / (2 * wi.g["L"]) * (c + 1))
                      * rng.standard_normal() for c in range(5)])
        srcs.append(list(s))
        flat.append(s)
    line.view("src").copy_(ctx.pack_r(flat, 5))
    line.deposit()
    Pg, rho = ol.deposit(srcs)
    assert rel(host(line.view("Pg")), Pg) < 1e-12
    assert rel(host(line.view("rho")), rho) < 1e-12
    line.close()
    p.close()
    ctx.close()


def _initial(ows, rng):
    states = []
    for wi in ows:
        nk = wi.g["nk"]
        C = np.diag(0.02 * rng.uniform(size=nk)).astype(complex)
        D = np.diag(0.02 * rng.uniform(size=nk)).astype(complex)
        P = 1e-4 * (rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk)))
        states.append([P, C, D])
    return states


def _coupled_setup(nks, wx, nx=512, dx=2e-9, seed=7):
    from pulsesuite_gb300.pstd import CoupledLine, Pstd1D, SheetSource
    ctx, ows = _wires(nks)
    p = Pstd1D(nx, dx, EPSR, n_abc=32, abc_strength=0.05)
    o = PO.Pstd1D(nx, dx, EPSR, n_abc=32, strength=0.05)
    tau = 5e-15
    w0 = (1.52 + 0.02) * O.E0 / O.HBAR
    src = SheetSource(index=60, E0=2e7, tau=tau, w0=w0, tpeak=0.0)
    line = CoupledLine(ctx, p, wx, source=src, t0=-0.5e-15)
    ol = PO.CoupledLine(o, ows, list(range(1, len(nks) + 1)), wx, src_index=60, E0=2e7, tau=tau,
                        w0=w0, tpeak=0.0, t0=-0.5e-15)
    rng = np.random.default_rng(seed)
    E = smooth_fields(rng, o.x, 2, 1e7)
    H = smooth_fields(rng, o.x, 2, 1e4)
    Ex = np.zeros(nx, complex)
    states = _initial(ows, rng)
    return ctx, ows, p, o, line, ol, E, H, Ex, states


def test_coupled_fp64_steps_vs_oracle():
    ctx, ows, p, o, line, ol, E, H, Ex, states = _coupled_setup([32, 32], [-20e-9, 30e-9])
    P = ctx.pack([s[0] for s in states])
    C = ctx.pack([s[1] for s in states])
    D = ctx.pack([s[2] for s in states])
    Eg, Hg, Exg = dev(E), dev(H), dev(Ex)
    dt = 0.01e-15
    for n in range(4):
        line.step(P, C, D, Eg, Hg, Exg, dt)
        E, H, Ex, _ = ol.step(states, E, H, Ex, dt)
    assert rel(host(Eg), E) < 1e-10
    assert rel(host(Hg), H) < 1e-10
    assert rel(host(Exg), Ex) < 1e-10
    assert np.abs(Ex).max() > 0
    for w in range(2):
        assert rel(host(ctx.mat(P, w)), states[w][0]) < 1e-10
        assert rel(host(ctx.mat(C, w)), states[w][1]) < 1e-10
        assert rel(host(ctx.mat(D, w)), states[w][2]) < 1e-10
    line.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_coupled_graph_replay_equals_direct(precision):
    ctx, ows, p, o, line, ol, E, H, Ex, states = _coupled_setup([32, 32], [-20e-9, 30e-9])
    dt = 0.01e-15

    def fresh():
        return (ctx.pack([s[0] for s in states]), ctx.pack([s[1] for s in states]),
                ctx.pack([s[2] for s in states]), dev(E), dev(H), dev(Ex))

    a = fresh()
    line.reset()
    for _ in range(3):
        line.step(*a, dt, precision=precision)
    b = fresh()
    g = line.graph(*b, dt, precision=precision)
    assert g.kernels > 20
    line.reset()
    b2 = fresh()
    for t, v in zip(b, b2):
        t.copy_(v)
    for _ in range(3):
        g.launch()
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    g.close()
    line.close()


def test_coupled_mixed_vs_fp64():
    ctx, ows, p, o, line, ol, E, H, Ex, states = _coupled_setup([64, 64], [-40e-9, 50e-9])
    dt = 0.01e-15

    def fresh():
        return (ctx.pack([s[0] for s in states]), ctx.pack([s[1] for s in states]),
                ctx.pack([s[2] for s in states]), dev(E), dev(H), dev(Ex))

    ref = fresh()
    line.reset()
    for _ in range(20):
        line.step(*ref, dt, precision=0)
    mix = fresh()
    line.reset()
    for _ in range(20):
        line.step(*mix, dt, precision=1)
    torch.cuda.synchronize()
    for w in range(2):
        assert rel(host(ctx.mat(mix[0], w)), host(ctx.mat(ref[0], w))) < 1e-5
        assert rel(np.diag(host(ctx.mat(mix[1], w))), np.diag(host(ctx.mat(ref[1], w)))) < 1e-5
    assert rel(host(mix[3]), host(ref[3])) < 1e-5
    line.close()
