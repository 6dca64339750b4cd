"""Contexts of wires with different Nk on the mixed path (needs a GPU).

The wires of one Nk form a bucket (contiguous in the packed layout); every GEMM kind of
a stage runs as one persistent launch over the jobs of all buckets, and the autotuner
picks the N tile of each bucket's exchange, commutator and source GEMMs.  Bars as for
one Nk: RHS relative error <= 1e-6 per wire, observables after a pulse segment <= 1e-5
against the FP64 path on the same context.
"""

import json

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import sbe_oracle as O  # noqa: E402

MAT = dict(me=0.067 * O.ME0, mh=0.45 * O.ME0, gap=1.52 * O.E0, HO=100e-3 * O.E0, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR,
           Gph=3e-3 * O.E0 / O.HBAR)
ALL = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
           LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)
# interleaved on purpose: the layout groups them into buckets 64 x2, 96 x2, 128 x2, 256
NKS = [64, 128, 96, 64, 256, 96, 128]
TEMPS = [300.0, 77.0, 150.0, 300.0, 200.0, 10.0, 250.0]


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pulsesuite_gb300 import build
    build.build()


def make_ctx(nks=NKS, temps=TEMPS):
    from pulsesuite_gb300.wires import WireContext, WireSpec
    specs = [WireSpec(nk=nk, L=np.pi / (3e9 / (nk / 2 - 0.5)), temp=t, wire_index=w + 1,
                      flags=dict(ALL), **MAT) for w, (nk, t) in enumerate(zip(nks, temps))]
    return WireContext(specs)


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


def test_layout_groups_wires_by_nk():
    ctx = make_ctx()
    order = sorted(range(len(NKS)), key=lambda w: (NKS[w], w))
    off = 0
    for w in order:
        assert ctx.mat_offset[w] == off
        off += NKS[w] ** 2
    assert ctx.total_mat == off
    ctx.close()


def _states(ctx, seed, pscale=1e-3):
    rng = np.random.default_rng(seed)
    st = [seeded(rng, nk, pscale) for nk in NKS]
    return st, [ctx.pack([s[i] for s in st]) for i in range(3)]


def test_uneven_rhs_vs_fp64():
    from pulsesuite_gb300 import _lib
    ctx = make_ctx()
    _, (P, C, D) = _states(ctx, 1)
    Ek = fields(ctx, [1e7 * (1 + 0.3 * w) for w in range(len(NKS))])
    r64 = ctx.rhs(P, C, D, Ek, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek, _lib.PREC_MIXED)
    ctx.check()
    assert [t[:2] for t in ctx.tiles()] == [(64, 2), (96, 2), (128, 2), (256, 1)]
    for a, b, n in zip(rmx, r64, ("dP", "dC", "dD")):
        for w in range(len(NKS)):
            e = rel(ctx.mat(a, w), ctx.mat(b, w))
            assert e < 1e-6, (n, w, NKS[w], e)
    ctx.close()


def _pulse_run(ctx, P, C, D, prec, nsteps=30, graph=False):
    from pulsesuite_gb300 import _lib  # noqa: F401
    nw = len(NKS)
    dt, tau = 0.1e-15, 30e-15
    amp = np.array([2e7 * (0.5 + 0.25 * w) for w in range(nw)])
    det = np.array([-10e-3 + 15e-3 * w for w in range(nw)]) * O.E0
    w0 = (1.52 * O.E0 + det) / O.HBAR
    src = ctx.zeros_r(5)

    def e(t):
        return amp * np.exp(-t * t / tau ** 2) * np.cos(w0 * t)

    Ek0 = fields(ctx, np.zeros(nw))
    dEk = fields(ctx, np.zeros(nw))
    g = None
    if graph:
        ctx.rk4_step(P.clone(), C.clone(), D.clone(), Ek0, dEk, dt, src.clone(), prec)
        g = ctx.rk4_graph(P, C, D, Ek0, dEk, dt, src, prec)
    for n in range(nsteps):
        t = -2 * tau + n * dt
        e0, e1 = e(t), e(t + dt)
        Ek0.copy_(fields(ctx, e0))
        dEk.copy_(fields(ctx, e1 - e0))
        if g is not None:
            g.launch()
        else:
            ctx.rk4_step(P, C, D, Ek0, dEk, dt, src, prec)
    torch.cuda.synchronize()
    if g is not None:
        g.close()
    ctx.check()
    return src


def test_uneven_rk4_pulse_vs_fp64():
    """30 RK4 steps of a pulse whose amplitude and detuning differ per wire."""
    from pulsesuite_gb300 import _lib
    ctx = make_ctx()
    st, _ = _states(ctx, 2, 1e-4)
    runs = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        P, C, D = (ctx.pack([s[i] for s in st]) for i in range(3))
        src = _pulse_run(ctx, P, C, D, prec)
        runs[prec] = (P, C, D, src)
    P64, C64, D64, s64 = runs[_lib.PREC_FP64]
    Pm, Cm, Dm, sm = runs[_lib.PREC_MIXED]
    for w in range(len(NKS)):
        assert rel(ctx.mat(Pm, w), ctx.mat(P64, w)) < 1e-5, w
        assert rel(ctx.mat(Cm, w).diagonal(), ctx.mat(C64, w).diagonal()) < 1e-5, w
        assert rel(ctx.mat(Dm, w).diagonal(), ctx.mat(D64, w).diagonal()) < 1e-5, w
        assert rel(ctx.rvec(sm, w, 5)[:3], ctx.rvec(s64, w, 5)[:3]) < 1e-5, w
    ctx.close()


def test_uneven_graph_replay_equals_direct():
    from pulsesuite_gb300 import _lib
    ctx = make_ctx()
    st, _ = _states(ctx, 3, 1e-4)
    out = []
    for graph in (False, True):
        P, C, D = (ctx.pack([s[i] for s in st]) for i in range(3))
        src = _pulse_run(ctx, P, C, D, _lib.PREC_MIXED, nsteps=3, graph=graph)
        out.append((P, C, D, src))
    for a, b in zip(*out):
        assert torch.isfinite(a).all()
        assert torch.equal(a, b)
    ctx.close()


def test_mixed_path_refuses_mixed_flags():
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.wires import WireContext, WireSpec
    L = np.pi / (3e9 / 31.5)
    ctx = WireContext([WireSpec(nk=64, L=L, wire_index=1, flags=dict(ALL), **MAT),
                       WireSpec(nk=64, L=L, wire_index=2, flags=dict(ALL, LF=False), **MAT)])
    P = ctx.zeros_state()
    with pytest.raises(_lib.SbeError, match="flags"):
        ctx.rhs(P, P, P, ctx.zeros_r(3), _lib.PREC_MIXED)
    ctx.close()


def _forced_cache(path, ctx, tile):
    """A cache file whose entry for this context's buckets forces one N tile."""
    data = json.loads(path.read_text())
    entry = data["entries"][0]
    for b in entry["buckets"]:
        b["exchange_bn"] = b["commutator_bn"] = b["sources_bn"] = tile
    lines = ["{\"sbe_autotune\": 1, \"entries\": [", json.dumps(entry), "]}"]
    path.write_text("\n".join(lines) + "\n")


def test_autotune_writes_loads_and_both_tiles_agree(tmp_path):
    from pulsesuite_gb300 import _lib
    cache = tmp_path / "tiles.json"
    ctx = make_ctx()
    tiles = ctx.autotune(cache)
    data = json.loads(cache.read_text())
    assert data["sbe_autotune"] == 1 and len(data["entries"]) == 1
    entry = data["entries"][0]
    assert [(b["nk"], b["nw"]) for b in entry["buckets"]] == [t[:2] for t in tiles]
    for b, t in zip(entry["buckets"], tiles):
        assert (b["exchange_bn"], b["commutator_bn"], b["sources_bn"], b["hh_split"]) == t[2:]
        assert all(v > 0 for k in ("exchange", "commutator", "sources") for v in b["ms"][k])
    _, (P, C, D) = _states(ctx, 4)
    Ek = fields(ctx, [2e7] * len(NKS))
    r64 = ctx.rhs(P, C, D, Ek, _lib.PREC_FP64)
    ctx.close()
    results = {}
    for tile in (128, 256):
        _forced_cache(cache, ctx, tile)
        c2 = make_ctx()
        assert all(t[2:5] == (tile, tile, tile) for t in c2.autotune(cache))   # loaded, not timed
        rmx = c2.rhs(P, C, D, Ek, _lib.PREC_MIXED)
        c2.check()
        for a, b in zip(rmx, r64):
            for w in range(len(NKS)):
                assert rel(c2.mat(a, w), c2.mat(b, w)) < 1e-6, (tile, w)
        results[tile] = rmx
        c2.close()
    # the N tile changes neither the K order nor the operands of any product
    for a, b in zip(results[128], results[256]):
        assert torch.equal(a, b)
