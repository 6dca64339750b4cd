"""The mixed path against the FP64 GPU path on the stated workloads (needs a GPU).

Bars: RHS relative Frobenius error <= 1e-6; end-of-pulse carrier densities n_e(k),
n_h(k) (diagonals of C, D) and the polarisation P <= 1e-5 relative to the FP64 run.

* Local-field wire (one GaAs-like wire, Nk = 64, T = 77 K, E0 = 1e6 V/m, tau = 100 fs,
  hbar w0 = Eg + 20 meV, RK4 dt = 0.1 fs, 4000 steps from t = -2 tau), and the one-shot
  RHS on the seeded state of that workload (Hermitian C, D with eigenvalues U[0, 0.1]
  from seeds 0 and 1, P complex normal with sigma = 1e-3 from seed 2) at 77 K.
* One wire (Nk = 256) at the centre of a 1-D PSTD grid of 8192 cells of 10 nm, the pulse
  (E0 = 1e7 V/m) launched from the left boundary, 20000 steps of 0.05 fs; the wire
  switches on when the field on it first exceeds 1e-3 E0 (the reference's gate), and
  the default run compares the first 5500 coupled steps from there (SBE_LONG_TESTS=1:
  every step to 20000).
* The RHS at Nk = 512 and 1024 on a weakly and a strongly excited state (the states a
  pulse E0 = 5e7 V/m, tau = 50 fs, T = 300 K drives in 200 and 2200 steps of 0.05 fs
  from t = -2 tau).
"""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import sbe_oracle as O  # noqa: E402

KB = 1.380649e-23
MAT = dict(me=0.067 * O.ME0, mh=0.45 * O.ME0, gap=1.52 * O.E0, HO=100e-3 * O.E0, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR,
           Gph=3e-3 * O.E0 / O.HBAR)
FLAGS = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
             LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)
W0 = (1.52 + 0.020) * O.E0 / O.HBAR


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pulsesuite_gb300 import build
    build.build()


def make_ctx(nk, temp, nw=1):
    from pulsesuite_gb300.wires import WireContext, WireSpec
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    specs = [WireSpec(nk=nk, L=L, temp=temp, wire_index=w + 1, flags=dict(FLAGS), **MAT)
             for w in range(nw)]
    return WireContext(specs)


def rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def fermi_state(ctx, temp):
    """P = 0 and C = D = diag(f(Ee + gap/2)) (the reference's initial occupations)."""
    P = ctx.zeros_state()
    ds = []
    for w in range(ctx.nw):
        Ee = ctx.table(w, "Ee").cpu().numpy()
        x = np.minimum((Ee + MAT["gap"] / 2.0) / (KB * temp), 700.0)
        ds.append(np.diag(1.0 / (np.exp(x) + 1.0)).astype(complex))
    return P, ctx.pack(ds), ctx.pack(ds)


def field_basis(ctx):
    """Per wire (0, FFTG(window), 0): a uniform Ey of unit amplitude in wire k space."""
    parts = []
    for w in range(ctx.nw):
        wk = ctx.table(w, "window_k")
        z = torch.zeros_like(wk)
        parts.append(torch.stack([z, wk, z]))
    return ctx.pack_r(parts, 3)


def pulse(t, E0, tau):
    return E0 * np.exp(-t * t / tau ** 2) * np.cos(W0 * t)


def run_local(ctx, state, prec, E0, tau, dt, t0, nsteps, snapshots=()):
    """nsteps RK4 steps of the local field E0 exp(-t^2/tau^2) cos(w0 t) from t0, through
    one captured step replayed with its field buffers refreshed every step."""
    from pulsesuite_gb300 import _lib
    P, C, D = state
    base = field_basis(ctx)
    Ek0 = torch.zeros_like(base)
    dEk = torch.zeros_like(base)
    src = ctx.zeros_r(5)
    # one direct step first (the mixed workspace exists before the capture)
    Pw, Cw, Dw = P.clone(), C.clone(), D.clone()
    ctx.rk4_step(Pw, Cw, Dw, Ek0, dEk, dt, src.clone(), prec)
    g = ctx.rk4_graph(P, C, D, Ek0, dEk, dt, src, prec)
    snaps = {}
    for n in range(nsteps):
        t = t0 + n * dt
        e0, e1 = pulse(t, E0, tau), pulse(t + dt, E0, tau)
        torch.mul(base, e0, out=Ek0)
        torch.mul(base, e1 - e0, out=dEk)
        g.launch()
        if n + 1 in snapshots:
            snaps[n + 1] = (P.clone(), C.clone(), D.clone())
    torch.cuda.synchronize()
    g.close()
    ctx.check()
    return snaps


def test_local_wire_nk64_77k_end_of_pulse():
    """4000 RK4 steps of 0.1 fs through the whole pulse (t = -200 fs ... +200 fs)."""
    from pulsesuite_gb300 import _lib
    ctx = make_ctx(64, 77.0)
    out = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        st = fermi_state(ctx, 77.0)
        run_local(ctx, st, prec, 1e6, 100e-15, 0.1e-15, -200e-15, 4000)
        out[prec] = st
    P64, C64, D64 = out[_lib.PREC_FP64]
    Pm, Cm, Dm = out[_lib.PREC_MIXED]
    ne64, nh64 = ctx.mat(C64, 0).diagonal(), ctx.mat(D64, 0).diagonal()
    assert float(ne64.real.max()) > 0 and float(P64.abs().max()) > 0
    errs = dict(ne=rel(ctx.mat(Cm, 0).diagonal(), ne64), nh=rel(ctx.mat(Dm, 0).diagonal(), nh64),
                P=rel(Pm, P64))
    print("local wire Nk=64 77 K, end of pulse:", errs)
    for k, e in errs.items():
        assert e < 1e-5, (k, e)
    ctx.close()


def seeded_one_shot(nk):
    def herm(seed):
        rng = np.random.default_rng(seed)
        z = (rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk))) / np.sqrt(2)
        q, _ = np.linalg.qr(z)
        return (q * rng.uniform(0.0, 0.1, nk)) @ q.conj().T
    rng = np.random.default_rng(2)
    P = 1e-3 * (rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk))) / np.sqrt(2)
    return P, herm(0), herm(1)


def test_one_shot_rhs_nk64_77k():
    """The seeded one-shot state at T = 77 K, field at the pulse peak (E0 = 1e6 V/m)."""
    from pulsesuite_gb300 import _lib
    ctx = make_ctx(64, 77.0)
    P, C, D = (ctx.pack([m]) for m in seeded_one_shot(64))
    Ek = field_basis(ctx) * 1e6
    r64 = ctx.rhs(P, C, D, Ek, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek, _lib.PREC_MIXED)
    ctx.check()
    errs = [rel(a, b) for a, b in zip(rmx, r64)]
    print("one-shot RHS Nk=64 77 K (dP, dC, dD):", errs)
    assert max(errs) < 1e-6, errs
    ctx.close()


@pytest.fixture(scope="module")
def driven_states():
    """Per Nk, the states after 200 (weak) and 2200 (strong) mixed RK4 steps of a pulse
    E0 = 5e7 V/m, tau = 50 fs at 300 K from t = -2 tau, with the field at that time."""
    from pulsesuite_gb300 import _lib
    out = {}
    for nk in (512, 1024):
        ctx = make_ctx(nk, 300.0)
        st = fermi_state(ctx, 300.0)
        dt, tau, t0 = 0.05e-15, 50e-15, -100e-15
        snaps = run_local(ctx, st, _lib.PREC_MIXED, 5e7, tau, dt, t0, 2200,
                          snapshots=(200, 2200))
        for n, s in snaps.items():
            out[(nk, "weak" if n == 200 else "strong")] = (ctx, s, pulse(t0 + n * dt, 5e7, tau))
    return out


@pytest.mark.parametrize("nk", [512, 1024])
@pytest.mark.parametrize("kind", ["weak", "strong"])
def test_mixed_rhs_large_nk_driven_state(driven_states, nk, kind):
    from pulsesuite_gb300 import _lib
    ctx, (P, C, D), e = driven_states[(nk, kind)]
    Ek = field_basis(ctx) * e
    r64 = ctx.rhs(P, C, D, Ek, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek, _lib.PREC_MIXED)
    ctx.check()
    ne = float(ctx.mat(C, 0).diagonal().real.max())
    errs = [rel(a, b) for a, b in zip(rmx, r64)]
    print(f"RHS Nk={nk} {kind} (max n_e {ne:.3e}, |P| {float(P.abs().max()):.3e}) "
          f"dP, dC, dD: {errs}")
    # W - W^H cancels to a few percent of W, so the truncating FP32 chains of the hi*hi
    # products set dC and dD: with K parts of at most 128 (four at Nk = 512, eight at
    # Nk = 1024) they measure 5.8-7.8e-7 at Nk = 512 and 7.2-9.7e-7 at Nk = 1024
    # (four parts at Nk = 1024: 1.1-1.3e-6); dP stays near 6e-8 at every Nk
    assert errs[0] < 1e-7, errs
    assert max(errs) < 1e-6, errs


def _config1_run(window):
    """One Nk = 256 wire at the centre of 8192 cells of 10 nm, the pulse (E0 = 1e7 V/m,
    tau = 100 fs, peak leaving the source at 300 fs) launched by a current sheet next to
    the left absorbing layer, 20000 steps of 0.05 fs in all.  As in the reference's
    QWCalculator (SBEs.py:5826-5860) the wire stays off, and only the grid is stepped,
    until the field on the wire first exceeds 1e-3 E0; from there FP64 and mixed coupled
    runs start from the same grid state and run ``window`` steps (None: to step 20000)."""
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.pstd import CoupledLine, Pstd1D, SheetSource
    nx, dx, dt, total = 8192, 10e-9, 0.05e-15, 20000
    E0, tau, tpeak, i_src = 1e7, 100e-15, 300e-15, 144
    ctx = make_ctx(256, 77.0)
    grid = Pstd1D(nx, dx, MAT["epsr"], n_abc=128, abc_strength=0.05)
    x = grid.x.cpu().numpy()
    L = np.pi / (3e9 / 127.5)
    near = torch.as_tensor(np.abs(x) <= L, device="cuda")
    eta = np.sqrt(1.25663706127e-06 / (8.8541878188e-12 * MAT["epsr"]))
    jamp = -2.0 * E0 / (eta * dx)
    E, H = grid.zeros(2), grid.zeros(2)
    J = grid.zeros(2)
    n = 0
    while n < total:
        th = (n + 0.5) * dt
        a = (th - tpeak) / tau
        J[0, i_src] = jamp * np.exp(-a * a) * np.cos(W0 * (th - tpeak))
        grid.step(E, H, J, dt)
        n += 1
        if n % 100 == 0 and float(E[:, near].abs().max()) > 1e-3 * E0:
            break
    gate = n
    assert 5000 < gate < 15000, gate
    end = total if window is None else min(total, gate + window)
    src = SheetSource(index=i_src, E0=E0, tau=tau, w0=W0, tpeak=tpeak)
    line = CoupledLine(ctx, grid, [0.0], source=src, t0=0.0, longitudinal=True)
    out = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        P, C, D = fermi_state(ctx, 77.0)
        Ex = torch.zeros(nx, dtype=torch.complex128, device="cuda")
        st = (P, C, D, E.clone(), H.clone(), Ex)
        line.reset()
        line.set_step(gate)
        line.step(*st, dt, prec)                 # direct step first (workspace before capture)
        g = line.graph(*st, dt, prec)
        for _ in range(end - gate - 1):
            g.launch()
        torch.cuda.synchronize()
        g.close()
        ctx.check()
        out[prec] = st
    P64, C64, D64, E64 = out[_lib.PREC_FP64][:4]
    Pm, Cm, Dm, Em = out[_lib.PREC_MIXED][:4]
    assert float(P64.abs().max()) > 0 and float(ctx.mat(C64, 0).diagonal().real.max()) > 0
    errs = dict(ne=rel(ctx.mat(Cm, 0).diagonal(), ctx.mat(C64, 0).diagonal()),
                nh=rel(ctx.mat(Dm, 0).diagonal(), ctx.mat(D64, 0).diagonal()),
                P=rel(Pm, P64), E=rel(Em, E64))
    print(f"coupled wire Nk=256 on 8192 cells, gate at step {gate}, steps {gate}-{end}:", errs)
    line.close()
    grid.close()
    ctx.close()
    return errs


def test_coupled_wire_nk256_grid8192_pulse_window():
    """The first 5500 coupled steps after the wire switches on (the rising edge and the
    pulse peak, which crosses the wire about 5200 steps after the gate opens)."""
    for k, e in _config1_run(5500).items():
        assert e < 1e-5, (k, e)


@pytest.mark.skipif(not os.environ.get("SBE_LONG_TESTS"),
                    reason="the whole 20000-step run (about 15 min of FP64 steps): "
                           "set SBE_LONG_TESTS=1")
def test_coupled_wire_nk256_grid8192_end_of_pulse():
    """Every step to step 20000 (the pulse has passed the wire)."""
    for k, e in _config1_run(None).items():
        assert e < 1e-5, (k, e)
