"""3-D PSTD field step on the GPU against the oracle and the reference's ElongfromRho
(needs a GPU).  FP64 transforms: <= 1e-12 of the oracle; FP32 transforms (FP64 fields):
<= 1e-6 per curl, <= 1e-5 after a run of steps."""

import types

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import pstd_oracle as PO  # noqa: E402
from tests.conftest import golden  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pulsesuite_gb300 import build
    build.build()


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else a
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def dev(x):
    return torch.as_tensor(np.ascontiguousarray(x)).cuda()


def rand_fields(rng, n, scale=1.0):
    return scale * (rng.standard_normal((3,) + n) + 1j * rng.standard_normal((3,) + n))


@pytest.mark.parametrize("n", [(16, 8, 32), (8, 64, 16), (32, 16, 8)])
def test_grid_tables_match_oracle(n):
    from pulsesuite_gb300.pstd import Pstd3D
    d = (20e-9, 15e-9, 25e-9)
    g = Pstd3D(n, d, 12.9)
    o = PO.Pstd3D(n, d, 12.9)
    for a in range(3):
        assert np.array_equal(g.x[a].cpu().numpy(), o.x[a])
        assert np.array_equal(g.q[a].cpu().numpy(), o.q[a])
    g.close()


# FP32 transforms of (y, z) planes up to 16384 points run as three passes with the
# planes in shared memory, larger planes (2 x 256 x 128) as five axis passes
@pytest.mark.parametrize("fp32,tol", [(False, 1e-12), (True, 1e-6)])
@pytest.mark.parametrize("n", [(16, 8, 32), (8, 64, 16), (32, 16, 8), (2, 256, 128), (4, 2, 1024),
                               (1024, 2, 4)])
def test_curl_vs_oracle(n, fp32, tol):
    from pulsesuite_gb300.pstd import Pstd3D
    d = (20e-9, 15e-9, 25e-9)
    g = Pstd3D(n, d, 12.9, fp32_work=fp32)
    o = PO.Pstd3D(n, d, 12.9)
    F = rand_fields(np.random.default_rng(sum(n)), n)
    got = g.curl(dev(F))
    torch.cuda.synchronize()
    assert rel(got, o.curl(F)) < tol
    g.close()


@pytest.mark.parametrize("fp32,tol", [(False, 1e-11), (True, 1e-5)])
def test_steps_with_current_and_absorber_vs_oracle(fp32, tol):
    from pulsesuite_gb300.pstd import Pstd3D
    n, d, epsr = (32, 16, 16), (20e-9, 20e-9, 20e-9), 12.9
    g = Pstd3D(n, d, epsr, n_abc=(4, 2, 3), abc_strength=0.05, fp32_work=fp32)
    o = PO.Pstd3D(n, d, epsr, n_abc=(4, 2, 3), strength=0.05)
    rng = np.random.default_rng(5)
    X = np.meshgrid(*o.x, indexing="ij")
    env = np.exp(-(X[0] ** 2 + X[1] ** 2 + X[2] ** 2) / (80e-9) ** 2)
    E = rand_fields(rng, n, 1e6) * env
    H = rand_fields(rng, n, 1e3) * env
    J = rand_fields(rng, n, 1e9) * env
    dt = 0.8 * g.max_dt()
    Eg, Hg, Jg = dev(E), dev(H), dev(J)
    E2, H2 = Eg.clone(), Hg.clone()
    for _ in range(10):
        g.step(Eg, Hg, Jg, dt)
        E, H = o.step(E, H, J, dt)
        # the two half-steps called one by one: with FP32 planes the fused step hands
        # the new H's transform from the H update to the E update, bit for bit the same
        g.update_h(E2, H2, dt)
        g.update_e(E2, H2, Jg, dt)
    torch.cuda.synchronize()
    assert rel(Eg, E) < tol and rel(Hg, H) < tol
    assert torch.equal(Eg, E2) and torch.equal(Hg, H2)
    g.close()


def test_step_rejects_unstable_dt():
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.pstd import Pstd3D
    g = Pstd3D((8, 8, 8), (10e-9,) * 3, 12.9)
    E, H = g.zeros(), g.zeros()
    with pytest.raises(_lib.SbeError, match="stability"):
        g.step(E, H, None, 1.01 * g.max_dt())
    g.close()


def test_elong_from_rho_matches_reference():
    """rhoPJ.ElongfromRho drop-in (the reference's centred k tables and its epsr rule)
    against the reference's outputs, P replaced by its transform as the reference does."""
    from pulsesuite_gb300 import rhoPJ
    g = golden("pstd3d")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    space = types.SimpleNamespace(Dims=3, Nx=nx, Ny=ny, Nz=nz, dx=float(g["dx"]),
                                  dy=float(g["dy"]), dz=float(g["dz"]), epsr=12.9)
    P = [g["Px"].copy(), g["Py"].copy(), g["Pz"].copy()]
    outs = [np.zeros((nx, ny, nz), complex) for _ in range(10)]
    rhoPJ.ElongfromRho(space, g["rho"].copy(), *P, *outs)
    names = ("ExlfromPRho", "EylfromPRho", "EzlfromPRho", "ExlfromP", "EylfromP", "EzlfromP",
             "ExlfromRho", "EylfromRho", "EzlfromRho", "RhoBound")
    for nm, a in zip(names, outs):
        assert rel(a, g[nm]) < 1e-13, nm
    for a, nm in zip(P, ("Pk_x", "Pk_y", "Pk_z")):
        assert rel(a, g[nm]) < 1e-13, nm


def test_full_size_grid_plane_wave_dispersion():
    """The 256 x 128 x 128 x 20 nm grid with FP32 transforms: a plane wave along x
    advances by the leapfrog's discrete phase, sin(w dt / 2) = v q dt / 2."""
    from pulsesuite_gb300.pstd import Pstd3D
    n, d, epsr = (256, 128, 128), (20e-9,) * 3, 12.9
    g = Pstd3D(n, d, epsr, fp32_work=True)
    x = g.x[0].cpu().numpy()
    v = PO.C0 / np.sqrt(epsr)
    dt = 0.5 * g.max_dt()
    kx = 2 * np.pi * 7 / (n[0] * d[0])
    w = 2.0 / dt * np.arcsin(v * kx * dt / 2.0)
    eta = np.sqrt(PO.MU0 / (PO.EPS0 * epsr))
    line = np.exp(1j * kx * x)
    E = torch.zeros((3,) + n, dtype=torch.complex128, device="cuda")
    H = torch.zeros_like(E)
    E[1] = dev(line)[:, None, None]
    hfac = np.exp(1j * w * dt / 2) * (v * kx * dt / 2) / np.sin(w * dt / 2) / eta
    H[2] = dev(line * hfac)[:, None, None]
    nsteps = 25
    for _ in range(nsteps):
        g.step(E, H, None, dt)
    torch.cuda.synchronize()
    want = line * np.exp(-1j * w * nsteps * dt)
    got = E[1, :, 37, 90].cpu().numpy()
    assert rel(got, want) < 1e-5
    assert float(E[0].abs().max()) < 1e-5 and float(E[2].abs().max()) < 1e-5
    g.close()


# ---- wires along z on the 3-D grid -------------------------------------------

from oracle import sbe_oracle as O  # noqa: E402

MAT = dict(me=0.067 * O.ME0, mh=0.45 * O.ME0, gap=1.52 * O.E0, HO=100e-3 * O.E0, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR,
           Gph=3e-3 * O.E0 / O.HBAR)
ALL = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
           LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)


def _grid3_setup(nks, wxy, fp32=False):
    from pulsesuite_gb300.pstd import CoupledGrid3, Pstd3D, SheetSource
    from pulsesuite_gb300.wires import WireContext, WireSpec
    n, d, epsr = (16, 16, 32), (20e-9, 20e-9, 5e-9), 12.9
    Ls = [np.pi / (3e9 / (nk / 2 - 0.5)) for nk in nks]
    ctx = WireContext([WireSpec(nk=nk, L=L, temp=300.0, wire_index=w + 1, flags=dict(ALL), **MAT)
                       for w, (nk, L) in enumerate(zip(nks, Ls))])
    ows = [O.Wire(nk, L, MAT, ALL, temp=300.0) for nk, L in zip(nks, Ls)]
    g = Pstd3D(n, d, epsr, n_abc=(3, 3, 4), abc_strength=0.05, fp32_work=fp32)
    o = PO.Pstd3D(n, d, epsr, n_abc=(3, 3, 4), strength=0.05)
    w0 = (1.52 + 0.02) * O.E0 / O.HBAR
    src = SheetSource(index=4, E0=2e7, tau=5e-15, w0=w0, tpeak=0.0)
    line = CoupledGrid3(ctx, g, wxy, source=src, pol=1, waist=60e-9, gate=12e-9, t0=-0.5e-15)
    ol = PO.CoupledGrid3(o, ows, range(1, len(nks) + 1), wxy, 12e-9, src_index=4, pol=1,
                         E0=2e7, tau=5e-15, w0=w0, tpeak=0.0, t0=-0.5e-15, waist=60e-9)
    rng = np.random.default_rng(9)
    X = np.meshgrid(*o.x, indexing="ij")
    env = np.exp(-(X[0] ** 2 + X[1] ** 2 + X[2] ** 2) / (60e-9) ** 2)
    E = rand_fields(rng, n, 1e6) * env
    H = np.zeros_like(E)
    states = []
    for nk in nks:
        C = np.diag(0.02 * rng.uniform(size=nk)).astype(complex)
        D = np.diag(0.02 * rng.uniform(size=nk)).astype(complex)
        P = 1e-4 * (rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk)))
        states.append([P, C, D])
    return ctx, g, line, o, ol, E, H, states


def test_grid3_sample_and_deposit_vs_oracle():
    ctx, g, line, o, ol, E, H, states = _grid3_setup([16, 24, 16],
                                                     [(-30e-9, 10e-9), (25e-9, -15e-9),
                                                      (5e-9, 40e-9)])
    line.sample(dev(E))
    ref = ol.sample(E)
    for w in range(3):
        got = ctx.rvec(line.view("Ek"), w, 3).cpu().numpy()
        for f in range(3):
            assert rel(got[f], ref[w][f]) < 1e-12, (w, f)
    rng = np.random.default_rng(3)
    srcs = []
    for w in range(3):
        nr = 2 * ctx.nk[w] + 2
        srcs.append((rng.standard_normal((5, nr)) + 1j * rng.standard_normal((5, nr))) * 1e-3)
    line.view("src").copy_(ctx.pack_r(srcs, 5))
    line.reset()
    dt = 0.01e-15
    line.deposit(dt)
    Pg, rho = ol.deposit([list(s) for s in srcs])
    J = ol.current(Pg, dt)
    torch.cuda.synchronize()
    assert rel(line.view("J"), J) < 1e-12
    assert rel(line.view("rho"), rho) < 1e-12
    g.close()


def test_grid3_coupled_fp64_steps_vs_oracle():
    ctx, g, line, o, ol, E, H, states = _grid3_setup([16, 24], [(-30e-9, 10e-9), (25e-9, -15e-9)])
    P = ctx.pack([s[0] for s in states])
    C = ctx.pack([s[1] for s in states])
    D = ctx.pack([s[2] for s in states])
    Eg, Hg = dev(E), dev(H)
    dt = 0.01e-15
    for _ in range(3):
        line.step(P, C, D, Eg, Hg, dt)
        E, H, _ = ol.step(states, E, H, dt)
    torch.cuda.synchronize()
    assert rel(Eg, E) < 1e-10 and rel(Hg, H) < 1e-10
    for w in range(2):
        for i in range(3):
            assert rel(ctx.mat((P, C, D)[i], w).cpu().numpy(), states[w][i]) < 1e-10, (w, i)
    g.close()


def test_grid3_graph_replay_and_mixed_vs_fp64():
    ctx, g, line, o, ol, E, H, states = _grid3_setup([16, 24], [(-30e-9, 10e-9), (25e-9, -15e-9)])
    dt = 0.01e-15

    def fresh():
        return (ctx.pack([s[0] for s in states]), ctx.pack([s[1] for s in states]),
                ctx.pack([s[2] for s in states]), dev(E), dev(H))

    runs = {}
    for prec in (0, 1):
        a = fresh()
        line.reset()
        line.step(*a, dt, precision=prec)
        gr = line.graph(*a, dt, precision=prec)
        for _ in range(9):
            gr.launch()
        torch.cuda.synchronize()
        gr.close()
        b = fresh()
        line.reset()
        for _ in range(10):
            line.step(*b, dt, precision=prec)
        torch.cuda.synchronize()
        for x, y in zip(a, b):
            assert torch.equal(x, y)
        runs[prec] = a
    ctx.check()
    for i in (0, 3):
        assert rel(runs[1][i], runs[0][i].cpu().numpy()) < 1e-5, i
    g.close()
