"""The PSTD oracle against the reference's golden vectors and the physics it must obey."""

import numpy as np

from oracle import pstd_oracle as PO
from oracle import sbe_oracle as O
from conftest import golden


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def test_grid_and_derivative_match_reference():
    g = golden("pstd")
    nx, dx = int(g["nx"]), float(g["dx"])
    x, q = PO.pstd_grid(nx, dx)
    assert np.array_equal(q, g["q"])
    assert np.array_equal(x, g["x_typespace"])
    assert np.array_equal(g["x_typespace"], g["x_helpers"])
    assert rel(PO.deriv(g["f"], g["q"]), g["df"]) < 1e-15


def test_longitudinal_formula_matches_reference():
    # The reference evaluates ElongfromRho with its centred kx table and epsr = 1
    # for an (Nx, 1, 1) grid; the restated formula reproduces it on those inputs.
    g = golden("pstd")
    e = PO.elong(g["rho"], g["px"], g["qx_space"], float(g["epsr_space"]))
    assert rel(e, g["Exl_PRho"]) < 1e-15


def test_spectral_derivative_is_exact_for_grid_modes():
    nx, dx = 512, 7e-9
    x, q = PO.pstd_grid(nx, dx)
    for m in (1, 5, 100):
        k = 2 * np.pi * m / (nx * dx)
        f = np.sin(k * x) + 1j * np.cos(2 * k * x)
        ref = k * np.cos(k * x) - 2j * k * np.sin(2 * k * x)
        assert rel(PO.deriv(f, q), ref) < 1e-12


def test_longitudinal_field_solves_gauss_law():
    nx, dx, epsr = 1024, 10e-9, 12.9
    x, q = PO.pstd_grid(nx, dx)
    k = 2 * np.pi * 3 / (nx * dx)
    rho = np.cos(k * x).astype(complex)
    Ex = PO.elong(rho, np.zeros(nx, complex), q, epsr)
    ref = np.sin(k * x) / (PO.EPS0 * epsr * k)
    assert rel(Ex, ref) < 1e-9          # q^2 + small in the denominator (rhoPJ.py:779)
    px = 1e-3 * np.sin(2 * k * x).astype(complex)
    Ex = PO.elong(np.zeros(nx, complex), px, q, epsr)
    assert rel(Ex, -px / (PO.EPS0 * epsr)) < 1e-9


def test_leapfrog_invariant_and_dispersion():
    nx, dx, epsr = 256, 10e-9, 12.9
    p = PO.Pstd1D(nx, dx, epsr)
    dt = 0.9 * 2 * dx * np.sqrt(epsr) / (PO.C0 * np.pi)
    assert PO.stable(dt, dx, epsr) and not PO.stable(1.2 * dt / 0.9, dx, epsr)
    rng = np.random.default_rng(0)
    E = np.zeros((2, nx), complex)
    H = np.zeros((2, nx), complex)
    for m in range(1, 20):
        k = 2 * np.pi * m / (nx * dx)
        E[0] += rng.standard_normal() * np.exp(1j * k * p.x)
        E[1] += rng.standard_normal() * np.cos(k * p.x)
    Hp = H
    H1 = p.update_h(E, H, dt)
    w0 = p.energy(E, Hp, H1)
    for _ in range(60):
        E = p.update_e(E, H1, None, dt)
        H2 = p.update_h(E, H1, dt)
        assert abs(p.energy(E, H1, H2) - w0) < 1e-12 * w0
        H1 = H2
    # one grid mode: the discrete leapfrog frequency sin(w dt / 2) = v q dt / 2
    m = 7
    k = 2 * np.pi * m / (nx * dx)
    v = PO.C0 / np.sqrt(epsr)
    wn = 2.0 / dt * np.arcsin(v * k * dt / 2.0)
    eta = np.sqrt(PO.MU0 / (PO.EPS0 * epsr))
    E = np.zeros((2, nx), complex)
    E[0] = np.exp(1j * k * p.x)
    H = np.zeros((2, nx), complex)
    H[0] = np.exp(1j * (k * p.x + wn * dt / 2)) / eta * (np.sin(wn * dt / 2) / (v * k * dt / 2))
    nsteps = 200
    for _ in range(nsteps):
        E, H = p.step(E, H, None, dt)
    # right-moving wave exp(i (k x - w t)) up to the exact discrete amplitude ratio
    ref = np.exp(1j * (k * p.x - wn * nsteps * dt))
    assert rel(E[0], ref) < 1e-9


def test_absorbing_layer_removes_outgoing_pulse():
    nx, dx, epsr = 1024, 10e-9, 12.9
    p = PO.Pstd1D(nx, dx, epsr, n_abc=96, strength=0.05)
    dt = 0.05e-15
    x = p.x
    v = PO.C0 / np.sqrt(epsr)
    eta = np.sqrt(PO.MU0 / (PO.EPS0 * epsr))
    w = 300e-9
    E = np.zeros((2, nx), complex)
    H = np.zeros((2, nx), complex)
    E[0] = np.exp(-(x / w) ** 2)
    H[0] = np.exp(-((x + v * dt / 2) / w) ** 2) / eta   # right-moving pulse, H at -dt/2
    e0 = np.sum(np.abs(E) ** 2)
    for _ in range(int(2.0 * nx * dx / (v * dt))):
        E, H = p.step(E, H, None, dt)
    assert np.sum(np.abs(E) ** 2) < 1e-4 * e0


def test_vectorised_spline_equals_reference_loop():
    rng = np.random.default_rng(3)
    x0 = np.linspace(-1e-7, 1.3e-7, 57)
    z0 = rng.standard_normal(57) + 1j * rng.standard_normal(57)
    x1 = np.concatenate([np.linspace(-1.2e-7, 1.5e-7, 91), x0[[0, -1]]])
    b, c, d = O.spline_coeffs(x0, z0)
    assert np.array_equal(PO.rescale_vec(x0, b, c, d, z0, x1), O.rescale_1d(x0, z0, x1))


def test_sheet_source_launches_incident_amplitude():
    nx, dx, epsr = 2048, 10e-9, 12.9
    p = PO.Pstd1D(nx, dx, epsr, n_abc=128, strength=0.05)
    dt = 0.05e-15
    tau, w0 = 10e-15, 2 * np.pi * PO.C0 / 800e-9
    line = PO.CoupledLine(p, [], [], [], src_index=200, E0=1.0, tau=tau, w0=w0,
                          tpeak=3 * tau)
    E = np.zeros((2, nx), complex)
    H = np.zeros((2, nx), complex)
    nsteps = int(8 * tau / dt)
    peak = 0.0
    for _ in range(nsteps):
        J = line.current(np.zeros((3, nx), complex), dt)
        line.n += 1
        E, H = p.step(E, H, J, dt)
        peak = max(peak, abs(E[0, 400].real))
    assert 0.97 < peak < 1.03


# ---- 3-D grid ---------------------------------------------------------------

def test_elong3d_matches_reference():
    """rhoPJ.ElongfromRho on a 3-D grid with the reference's own (centred) k tables:
    all ten outputs and the transformed P it leaves in its inputs."""
    g = golden("pstd3d")
    e_prho, e_p, e_rho, rho_b, pk = PO.elong3d(g["rho"], g["Px"], g["Py"], g["Pz"], g["qx"],
                                               g["qy"], g["qz"], float(g["epsr"]))
    for c, ax in enumerate("xyz"):
        assert rel(e_prho[c], g[f"E{ax}lfromPRho"]) < 1e-14
        assert rel(e_p[c], g[f"E{ax}lfromP"]) < 1e-14
        assert rel(e_rho[c], g[f"E{ax}lfromRho"]) < 1e-14
        assert rel(pk[c], g[f"Pk_{ax}"]) < 1e-14
    assert rel(rho_b, g["RhoBound"]) < 1e-14


def test_qspace_derivatives_and_3d_axes_match_reference():
    """usefulsubs.py:233-380: the q-space derivative is f (i q) along the axis; the
    FFT derivative of a 2-D array along y; the axes of the 256 x 128 x 128 x 20 nm grid."""
    g = golden("pstd3d")
    f1, f2, qa, qb = g["f1"], g["f2"], g["qa"], g["qb"]
    assert np.array_equal(f1 * (1j * qa), g["dfdx1D_q"])
    assert np.array_equal(f1 * (1j * qa), g["dfdy1D_q"])
    assert np.array_equal(f2 * (1j * qa)[:, None], g["dfdx2D_q"])
    assert np.array_equal(f2 * (1j * qb)[None, :], g["dfdy2D_q"])
    d = np.stack([PO.deriv(f2[i], qb) for i in range(f2.shape[0])])
    assert rel(d, g["dfdy2D"]) < 1e-15
    for ax, n in (("x", 256), ("y", 128), ("z", 128)):
        x, q = PO.pstd_grid(n, 20e-9)
        assert np.array_equal(x, g[f"grid_{ax}"])
        assert np.array_equal(q, g[f"q_{ax}"])


def _plane_wave3(p, kvec, pol):
    """E, H of a plane wave exp(i k.r) with E along pol (pol . k = 0)."""
    X = np.meshgrid(*p.x, indexing="ij")
    phase = np.exp(1j * sum(k * xx for k, xx in zip(kvec, X)))
    E = np.stack([pol[c] * phase for c in range(3)])
    return E


def test_curl3d_of_grid_modes_and_divergence_free():
    n, d = (16, 12, 10), (7e-9, 9e-9, 11e-9)
    p = PO.Pstd3D(n, d, 12.9)
    m = (2, 1, 3)
    kvec = [2 * np.pi * mm / (nn * dd) for mm, nn, dd in zip(m, n, d)]
    pol = np.cross(kvec, [0.3, -1.0, 0.7])
    E = _plane_wave3(p, kvec, pol)
    want = np.stack([1j * np.cross(kvec, pol)[c] * E[c] / pol[c] for c in range(3)])
    assert rel(p.curl(E), want) < 1e-12
    # div curl = 0 in k space
    rng = np.random.default_rng(0)
    F = rng.standard_normal((3,) + n) + 1j * rng.standard_normal((3,) + n)
    ck = [np.fft.fftn(c) for c in p.curl(F)]
    div = p.Q[0] * ck[0] + p.Q[1] * ck[1] + p.Q[2] * ck[2]
    qmax = max(np.abs(q).max() for q in p.q)
    assert np.abs(div).max() < 1e-12 * qmax * max(np.abs(c).max() for c in ck)


def test_leapfrog3d_invariant_and_dispersion():
    n, d, epsr = (16, 16, 8), (10e-9, 10e-9, 10e-9), 12.9
    p = PO.Pstd3D(n, d, epsr)
    v = PO.C0 / np.sqrt(epsr)
    # stable for v dt |q|max / 2 <= 1 with |q|max = sqrt(3) pi / dx
    dt = 0.3 * d[0] / v
    rng = np.random.default_rng(1)
    E = rng.standard_normal((3,) + n) + 1j * rng.standard_normal((3,) + n)
    H = 1e-3 * (rng.standard_normal((3,) + n) + 1j * rng.standard_normal((3,) + n))
    Hn = p.update_h(E, H, dt)
    e0 = p.energy(E, H, Hn)
    H = Hn
    for _ in range(50):
        E = p.update_e(E, H, None, dt)
        Hn = p.update_h(E, H, dt)
        e1 = p.energy(E, H, Hn)
        H = Hn
    assert abs(e1 - e0) < 1e-10 * abs(e0)
    # a plane wave along x advances by the discrete phase: sin(w dt / 2) = v q dt / 2
    kx = 2 * np.pi * 3 / (n[0] * d[0])
    pol = np.array([0.0, 1.0, 0.0])
    E = _plane_wave3(p, [kx, 0.0, 0.0], pol)
    w = 2.0 / dt * np.arcsin(v * kx * dt / 2.0)
    eta = np.sqrt(PO.MU0 / (PO.EPS0 * epsr))
    H = np.stack([0 * E[0], 0 * E[0], E[1] / eta * np.exp(1j * w * dt / 2) *
                  (v * kx * dt / 2) / np.sin(w * dt / 2)])
    nsteps = 20
    for _ in range(nsteps):
        E, H = p.step(E, H, None, dt)
    want = _plane_wave3(p, [kx, 0.0, 0.0], pol) * np.exp(-1j * w * nsteps * dt)
    assert rel(E, want) < 1e-9
