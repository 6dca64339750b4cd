"""Mixed-precision (tcgen05) RHS and RK4 step vs the FP64 GPU path (needs a GPU).

Accuracy bars of the mixed path: RHS relative Frobenius error <= 1e-6;
observables after a pulse segment <= 1e-5 relative to the FP64 run.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import sbe_oracle as O  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pulsesuite_gb300 import build
    build.build()


MAT = dict(me=0.067 * O.ME0, mh=0.45 * O.ME0, gap=1.52 * O.E0, HO=100e-3 * O.E0, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR,
           Gph=3e-3 * O.E0 / O.HBAR)
ALL = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
           LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)


def make_ctx(nk, nw, temp=300.0, flags=None, edc=0.0):
    from pulsesuite_gb300.wires import WireContext, WireSpec
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    specs = [WireSpec(nk=nk, L=L, temp=temp, wire_index=w + 1, flags=dict(flags or ALL),
                      Edc=edc, **MAT) for w in range(nw)]
    return WireContext(specs), L


def seeded(rng, nk, pscale=1e-3):
    def herm(scale):
        z = rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk))
        q, _ = np.linalg.qr(z)
        return (q * rng.uniform(0, scale, nk)) @ q.conj().T
    P = pscale * (rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk))) / np.sqrt(2)
    return P, herm(0.1), herm(0.1)


def fields(ctx, amps):
    out = []
    for w, a in enumerate(amps):
        wk = ctx.table(w, "window_k").cpu().numpy()
        z = np.zeros_like(wk)
        out.append(np.stack([z, a * wk, z]))
    return ctx.pack_r(out, 3)


def rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


# 16 and 32: one K block (the first split-K half of W and V is empty); 48, 96: an
# uneven split of two and three K blocks
@pytest.mark.parametrize("nk", [16, 32, 48, 64, 96, 128, 256])
def test_mixed_rhs_vs_fp64(nk):
    from pulsesuite_gb300 import _lib
    nw = 3
    ctx, _ = make_ctx(nk, nw)
    rng = np.random.default_rng(nk)
    st = [seeded(rng, nk) for _ in range(nw)]
    P = ctx.pack([s[0] for s in st])
    C = ctx.pack([s[1] for s in st])
    D = ctx.pack([s[2] for s in st])
    Ek = fields(ctx, [1e7, 3e7, 5e6])
    r64 = ctx.rhs(P, C, D, Ek, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek, _lib.PREC_MIXED)
    ctx.check()
    for a, b, n in zip(rmx, r64, ("dP", "dC", "dD")):
        for w in range(nw):
            e = rel(ctx.mat(a, w), ctx.mat(b, w))
            assert e < 1e-6, (nk, n, w, e)


def test_bounded_wait_gives_up_and_context_stays_usable():
    """A bounded device wait that nothing satisfies gives up (no hang, no fault), the
    next check reports SBE_ERR_TIMEOUT once, and the context then computes as before."""
    from pulsesuite_gb300 import _lib
    nk, nw = 64, 2
    ctx, _ = make_ctx(nk, nw)
    rng = np.random.default_rng(5)
    st = [seeded(rng, nk) for _ in range(nw)]
    P = ctx.pack([s[0] for s in st])
    C = ctx.pack([s[1] for s in st])
    D = ctx.pack([s[2] for s in st])
    Ek = fields(ctx, [1e7, 2e7])
    before = ctx.rhs(P, C, D, Ek, _lib.PREC_MIXED)
    ctx.check()
    assert ctx.wait_selftest()
    with pytest.raises(_lib.SbeError) as e:
        ctx.check()
    assert "(code 5)" in str(e.value)   # SBE_ERR_TIMEOUT
    ctx.check()                # the flag was cleared
    after = ctx.rhs(P, C, D, Ek, _lib.PREC_MIXED)
    ctx.check()
    for a, b in zip(after, before):
        assert torch.equal(a, b)


@pytest.mark.parametrize("prec", [0, 1])
def test_graph_replay_matches_direct_step(prec):
    """A captured RK4 step replays to the same state as the direct call."""
    nk, nw = 64, 2
    ctx, _ = make_ctx(nk, nw)
    rng = np.random.default_rng(11)
    st = [seeded(rng, nk) for _ in range(nw)]
    Ek0 = fields(ctx, [1e7, 2e7])
    dEk = fields(ctx, [1e5, -1e5])
    outs = []
    for use_graph in (False, True):
        P = ctx.pack([s[0] for s in st])
        C = ctx.pack([s[1] for s in st])
        D = ctx.pack([s[2] for s in st])
        src = ctx.zeros_r(5)
        if use_graph:
            ctx.rk4_step(P.clone(), C.clone(), D.clone(), Ek0, dEk, 1e-16, src.clone(), prec)
            g = ctx.rk4_graph(P, C, D, Ek0, dEk, 1e-16, src, prec)
            assert g.kernels > 10
            g.launch()
            g.close()
        else:
            ctx.rk4_step(P, C, D, Ek0, dEk, 1e-16, src, prec)
        torch.cuda.synchronize()
        outs.append((P, C, D, src))
    for a, b in zip(*outs):
        assert torch.isfinite(a).all()
        assert torch.equal(a, b)


def test_mixed_rejects_dc_transport():
    """DCTrans leaves C and D non-Hermitian (the reference's shift pairs the centred
    k array with the FFT's natural order); the mixed path's operands assume Hermitian
    C and D, so it refuses such a context and the FP64 path still steps it."""
    from pulsesuite_gb300 import _lib
    nk, nw = 64, 2
    ctx, _ = make_ctx(nk, nw, flags=dict(ALL, DCTrans=True), edc=5e7)
    st = [seeded(np.random.default_rng(4), nk, 1e-4) for _ in range(nw)]
    P = ctx.pack([s[0] for s in st])
    C = ctx.pack([s[1] for s in st])
    D = ctx.pack([s[2] for s in st])
    Ek = fields(ctx, [1e7, 2e7])
    src = ctx.zeros_r(5)
    with pytest.raises(_lib.SbeError, match="DCTrans"):
        ctx.rk4_step(P, C, D, Ek, Ek * 0, 0.1e-15, src, _lib.PREC_MIXED)
    C0 = C.clone()
    ctx.rk4_step(P, C, D, Ek, Ek * 0, 0.1e-15, src, _lib.PREC_FP64)
    ctx.check()
    assert torch.isfinite(C).all() and not torch.equal(C, C0)


@pytest.mark.parametrize("nk,ehs", [(64, False), (128, False), (64, True)])
def test_mixed_rk4_pulse_vs_fp64(nk, ehs):
    """40 RK4 steps through the rising edge of a pulse, mixed vs FP64 (with ehs: the
    carrier-carrier rates in the relaxation, FP32 kernel against the FP64 one)."""
    from pulsesuite_gb300 import _lib
    nw = 2
    ctx, _ = make_ctx(nk, nw, flags=dict(ALL, EHs=ehs))
    rng = np.random.default_rng(3)
    st = [seeded(rng, nk, 1e-4) for _ in range(nw)]
    states = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        P = ctx.pack([s[0] for s in st])
        C = ctx.pack([s[1] for s in st])
        D = ctx.pack([s[2] for s in st])
        src = ctx.zeros_r(5)
        dt = 0.1e-15
        tau = 30e-15
        w0 = (1.52 * O.E0 + 20e-3 * O.E0) / O.HBAR
        for n in range(40):
            t = -2 * tau + n * dt
            e0 = 2e7 * np.exp(-t * t / tau ** 2) * np.cos(w0 * t)
            t1 = t + dt
            e1 = 2e7 * np.exp(-t1 * t1 / tau ** 2) * np.cos(w0 * t1)
            Ek0 = fields(ctx, [e0, 0.5 * e0])
            dEk = fields(ctx, [e1 - e0, 0.5 * (e1 - e0)])
            ctx.rk4_step(P, C, D, Ek0, dEk, dt, src, prec)
        states[prec] = (P, C, D, src, ctx.charge())
    ctx.check()
    P64, C64, D64, s64, q64 = states[_lib.PREC_FP64]
    Pm, Cm, Dm, sm, qm = states[_lib.PREC_MIXED]
    # the FP64 conservation check of the last step sees the same carrier numbers
    assert rel(qm, q64) < 1e-5
    for w in range(nw):
        ne64 = ctx.mat(C64, w).diagonal()
        nem = ctx.mat(Cm, w).diagonal()
        assert rel(nem, ne64) < 1e-5
        assert rel(ctx.mat(Pm, w), ctx.mat(P64, w)) < 1e-5
        assert rel(ctx.rvec(sm, w, 5)[:3], ctx.rvec(s64, w, 5)[:3]) < 1e-5


def _deph_check(ctx, nks, C, D):
    De64, Dh64 = ctx.deph(C, D, fp32=False)
    De32, Dh32 = ctx.deph(C, D, fp32=True)
    ctx.check()
    off = 0
    for w, nk in enumerate(nks):
        rows = 2 * nk + 1
        n = rows * nk
        for a, b, name in ((De32, De64, "De"), (Dh32, Dh64, "Dh")):
            aw = a[off:off + n].reshape(rows, nk)
            bw = b[off:off + n].reshape(rows, nk)
            # the band structure (zeros where k + q leaves the grid) is exact
            assert torch.equal(aw == 0, bw == 0), (name, w)
            e = rel(aw, bw)
            assert e < 2e-6, (nk, name, w, e)
            # rows q and -q separately: a wrong mirror shows in one half only
            for half in (slice(0, nk), slice(nk + 1, rows)):
                assert rel(aw[half], bw[half]) < 2e-6, (nk, name, w, half)
        off += n


# 2 wires: the per-wire kernel; 6 and 20 identical wires: one group sharing its
# Lorentzian factors (chunks of 8 and 32 wires, partly filled)
@pytest.mark.parametrize("nk,nw", [(16, 2), (48, 2), (256, 2), (48, 6), (256, 20)])
def test_fp32_dephasing_sums_vs_fp64(nk, nw):
    """The mixed path's FP32 off-diagonal dephasing sums (rows -q formed from the
    sums of row q) against the FP64 reference loops, every row and wire."""
    ctx, _ = make_ctx(nk, nw)
    rng = np.random.default_rng(100 + nk + nw)
    st = [seeded(rng, nk) for _ in range(nw)]
    C = ctx.pack([s[1] for s in st])
    D = ctx.pack([s[2] for s in st])
    _deph_check(ctx, [nk] * nw, C, D)


def test_fp32_dephasing_mixed_groups():
    """Wires of two lengths and two masses: a group of five, a group of four and two
    single wires, interleaved in the context."""
    from pulsesuite_gb300.wires import WireContext, WireSpec
    nk = 48
    L0 = np.pi / (3e9 / (nk / 2 - 0.5))
    kinds = [0, 1, 0, 2, 0, 1, 0, 1, 3, 0, 1]
    specs = []
    for w, kd in enumerate(kinds):
        mat = dict(MAT)
        L = L0 * (1.25 if kd in (1, 3) else 1.0)
        if kd >= 2:
            mat["me"] = 0.07 * O.ME0 if kd == 2 else 0.06 * O.ME0
        specs.append(WireSpec(nk=nk, L=L, temp=300.0, wire_index=w + 1, flags=dict(ALL), **mat))
    ctx = WireContext(specs)
    rng = np.random.default_rng(7)
    st = [seeded(rng, nk) for _ in kinds]
    C = ctx.pack([s[1] for s in st])
    D = ctx.pack([s[2] for s in st])
    _deph_check(ctx, [nk] * len(kinds), C, D)
