"""CPU FP64 restatement of the 1-D PSTD field step and of its coupling to the wires.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/`` and by ``bench.py``'s CPU
baseline; nothing in ``pulsesuite_gb300`` imports or calls it.

The reference has no 1-D Maxwell stepper (rahulranjansah/pulsesuite,
``src/pulsesuite/...``); the step below assembles its pieces, each cited:

* grids: positions ``GetSpaceArray`` (PSTD3D/typespace.py:815-849, numpy linspace),
  wavenumbers in FFT order ``GetKArray`` (libpulsesuite/helpers.py:838-863);
* spectral derivative ``dfdx1D`` = IFFT(i q FFT f) (PSTD3D/usefulsubs.py:163-185);
* longitudinal field ``ElongfromRho`` (PSTD3D/rhoPJ.py:703-880), x component:
  small = (q[1] - q[0]) / 1e4 (:779), rho_term = -i rho / (eps (q^2 + small)),
  P_term = -(q Px) / (eps (q^2 + small)), Ex = IFFT((rho_term + P_term) q) (:836-866);
* absorbing mask multiply as in ``ApplyABC`` (usefulsubs.py:584-609), with the
  mask exp(-strength s^2) over n_abc cells at each end (s = depth fraction);
* leapfrog for propagation along x: d_t Hz = -(1/mu0) d_x Ey, d_t Hy = (1/mu0) d_x Ez,
  d_t Ey = -(1/eps)(d_x Hz + Jy), d_t Ez = (1/eps)(d_x Hy - Jz);
* field -> wire: ``Prop2QW`` (PSTD3D/qwoptics.py:667-715) with the grid spline
  evaluated at x_w + r; wire -> field: ``QW2Prop`` (qwoptics.py:717-805) of the
  real-space sources at x - x_w, summed over wires; Rho = RhoH - RhoE (SBEs.py:5917).
"""

import numpy as np

from . import sbe_oracle as O

MU0 = 1.25663706127e-06   # scipy.constants.mu_0 (CODATA 2022)
EPS0 = O.EPS0
C0 = 299792458.0


def pstd_grid(nx, dx):
    """Positions (typespace.py:815-849) and FFT-order wavenumbers (helpers.py:838-863)."""
    x = O.space_array(nx, (nx - 1) * dx)
    dq = 2.0 * np.pi / (nx * dx)
    i = np.arange(nx)
    q = np.where(i <= nx // 2, i, i - nx).astype(float) * dq
    return x, q


def abc_mask(nx, n_abc, strength):
    j = np.arange(nx)
    d = np.minimum(j, nx - 1 - j)
    m = np.ones(nx)
    if n_abc > 0:
        inl = d < n_abc
        s = (n_abc - d[inl]) / n_abc
        m[inl] = np.exp(-strength * s * s)
    return m


def deriv(f, q):
    """usefulsubs.py:163-185 dfdx1D."""
    return np.fft.ifft(np.fft.fft(np.asarray(f, complex)) * (1j * q))


def elong(rho, px, q, epsr):
    """rhoPJ.py:836-866 restricted to the x component."""
    small = (q[1] - q[0]) / 1e4
    inv_eps = 1.0 / (EPS0 * epsr)
    rk = np.fft.fft(np.asarray(rho, complex))
    pk = np.fft.fft(np.asarray(px, complex))
    qs = q * q + small
    rho_term = -1j * rk * inv_eps / qs
    p_term = -(q * pk) * inv_eps / qs
    return np.fft.ifft((rho_term + p_term) * q)


def stable(dt, dx, epsr):
    return C0 / np.sqrt(epsr) * dt * np.pi / dx <= 2.0


class Pstd1D:
    """Field state E = (Ey, Ez), H = (Hz, Hy) on the grid (2 x nx complex each)."""

    def __init__(self, nx, dx, epsr, n_abc=0, strength=0.0):
        self.nx, self.dx, self.epsr = nx, dx, epsr
        self.x, self.q = pstd_grid(nx, dx)
        self.mask = abc_mask(nx, n_abc, strength)
        self.masked = n_abc > 0

    def update_h(self, E, H, dt):
        a = dt / MU0
        H = H.copy()
        H[0] = H[0] + (-a) * deriv(E[0], self.q)
        H[1] = H[1] + a * deriv(E[1], self.q)
        if self.masked:
            H = H * self.mask
        return H

    def update_e(self, E, H, J, dt):
        ie = dt / (EPS0 * self.epsr)
        E = E.copy()
        E[0] = E[0] + (-ie) * deriv(H[0], self.q)
        E[1] = E[1] + ie * deriv(H[1], self.q)
        if J is not None:
            E[0] = E[0] + (-ie) * J[0]
            E[1] = E[1] + (-ie) * J[1]
        if self.masked:
            E = E * self.mask
        return E

    def step(self, E, H, J, dt):
        H = self.update_h(E, H, dt)
        return self.update_e(E, H, J, dt), H

    def energy(self, E, H_prev, H_next):
        """Discrete invariant of the leapfrog (no mask, no current):
        eps |E^n|^2 + mu0 Re(H^{n-1/2} . conj(H^{n+1/2})), summed over the grid."""
        e = EPS0 * self.epsr * np.sum(np.abs(E) ** 2)
        h = MU0 * np.sum(np.real(H_prev * np.conj(H_next)))
        return e + h


def rescale_vec(x0, b, c, d, z0, x1):
    """Vectorised spliner.py:153-189 evaluation with precomputed coefficients
    (locate = binary search, spliner.py:1137-1167; 0 outside [x0[0], x0[-1]])."""
    x1 = np.asarray(x1, float)
    out = np.zeros(len(x1), complex)
    n = len(x0)
    ok = (x1 >= x0[0]) & (x1 <= x0[n - 1])
    u = x1[ok]
    j = np.searchsorted(x0, u, side="right") - 1
    j = np.clip(j, 0, n - 1)
    dx = u - x0[j]
    z0 = np.asarray(z0, complex)
    out[ok] = z0[j] + dx * (b[j] + dx * (c[j] + dx * d[j]))
    return out


class CoupledLine:
    """Wires on the 1-D grid (one oracle ``Wire`` per wire, its 1-based index and
    centre position) with a soft-source current sheet at cell ``src_index``."""

    def __init__(self, pstd, wires, windex, wx, src_index=-1, E0=0.0, tau=1.0, w0=0.0,
                 tpeak=0.0, t0=0.0, longitudinal=True):
        self.p = pstd
        self.wires = wires
        self.windex = list(windex)
        self.wx = np.asarray(wx, float)
        self.src_index, self.E0, self.tau, self.w0, self.tpeak, self.t0 = (
            src_index, E0, tau, w0, tpeak, t0)
        self.longitudinal = longitudinal
        self.eta = np.sqrt(MU0 / (EPS0 * pstd.epsr))
        nx = pstd.nx
        self.Pold = np.zeros((3, nx), complex)
        self.n = 0

    def sample(self, Ex, E):
        """Grid fields at time t_n on every wire: [Ex_k, Ey_k, Ez_k] per wire."""
        x = self.p.x
        coefs = [O.spline_coeffs(x, f) for f in (Ex, E[0], E[1])]
        out = []
        for wi, xw in zip(self.wires, self.wx):
            u = xw + wi.g["r"]
            ek = []
            for f, (b, c, d) in zip((Ex, E[0], E[1]), coefs):
                v = rescale_vec(x, b, c, d, f, u) * wi.window
                ek.append(O.fftg(np.real(v).astype(complex)))
            out.append(ek)
        return out

    def deposit(self, srcs):
        """srcs: per wire real-space (Px, Py, Pz, re, rh).  Returns (Pg (3, nx), rho)."""
        x = self.p.x
        nx = self.p.nx
        Pg = np.zeros((3, nx), complex)
        rho = np.zeros(nx, complex)
        for wi, xw, s in zip(self.wires, self.wx, srcs):
            r = wi.g["r"]
            u = x - xw
            vals = []
            for comp in s:
                b, c, d = O.spline_coeffs(r, comp)
                vals.append(rescale_vec(r, b, c, d, comp, u))
            for k in range(3):
                Pg[k] = Pg[k] + vals[k]
            rho = rho + (vals[4] - vals[3])
        return Pg, rho

    def current(self, Pg, dt):
        J = np.zeros((2, self.p.nx), complex)
        J[0] = (Pg[1] - self.Pold[1]) / dt
        J[1] = (Pg[2] - self.Pold[2]) / dt
        if self.src_index >= 0:
            th = self.t0 + (self.n + 0.5) * dt
            a = (th - self.tpeak) / self.tau
            einc = np.exp(-a * a) * np.cos(self.w0 * (th - self.tpeak))
            jamp = -2.0 * self.E0 / (self.eta * self.p.dx)
            J[0, self.src_index] += jamp * einc
        self.Pold = Pg.copy()
        return J

    def step(self, states, E, H, Ex, dt):
        """states: per wire [P, C, D] (updated in place).  Returns (E, H, Ex, srcs)."""
        eks = self.sample(Ex, E)
        H = self.p.update_h(E, H, dt)
        srcs = []
        z = [np.zeros_like(eks[0][0])] * 3
        for i, (wi, st) in enumerate(zip(self.wires, states)):
            P, C, D, Px, Py, Pz, re, rh = wi.rk4_step(st[0], st[1], st[2], eks[i], z, dt,
                                                     self.windex[i])
            st[0], st[1], st[2] = P, C, D
            srcs.append([O.ifftg(a) for a in (Px, Py, Pz, re, rh)])
        Pg, rho = self.deposit(srcs)
        J = self.current(Pg, dt)
        E = self.p.update_e(E, H, J, dt)
        if self.longitudinal:
            Ex = elong(rho, Pg[0], self.p.q, self.p.epsr)
        self.n += 1
        return E, H, Ex, srcs


# ---------------------------------------------------------------------------
# 3-D grid (six field components on nx x ny x nz, C order, z fastest)


def elong3d(rho, Px, Py, Pz, qx, qy, qz, epsr):
    """rhoPJ.py:703-880 ElongfromRho on a 3-D grid, with the wavenumber tables the
    caller passes (the reference passes its centred GetKxArray/GetKyArray/GetKzArray,
    typespace.py:958-1030): small = (qx[1] - qx[0]) / 1e4 (:779); in k space
    rho_B = -i q.P, rho_term = -i rho / (eps (q^2 + small)), P_term = -(q.P) / (eps
    (q^2 + small)); the nine fields (rho + P, P, rho) x q_c and rho_B back in real space.
    Returns (E_PRho (3,..), E_P (3,..), E_Rho (3,..), RhoBound, P_k (3,..)), P_k being
    the transformed P that the reference leaves in its input arrays."""
    small = (qx[1] - qx[0]) / 1e4
    inv_eps = 1.0 / (EPS0 * epsr)
    rk = np.fft.fftn(np.asarray(rho, complex))
    pk = [np.fft.fftn(np.asarray(p, complex)) for p in (Px, Py, Pz)]
    QX, QY, QZ = np.meshgrid(qx, qy, qz, indexing="ij")
    qs = QX ** 2 + QY ** 2 + QZ ** 2 + small
    qdotp = QX * pk[0] + QY * pk[1] + QZ * pk[2]
    rho_b = -1j * qdotp
    rho_term = -1j * rk * inv_eps / qs
    p_term = -qdotp * inv_eps / qs
    q3 = (QX, QY, QZ)
    e_prho = np.stack([np.fft.ifftn((rho_term + p_term) * q) for q in q3])
    e_p = np.stack([np.fft.ifftn(p_term * q) for q in q3])
    e_rho = np.stack([np.fft.ifftn(rho_term * q) for q in q3])
    return e_prho, e_p, e_rho, np.fft.ifftn(rho_b), np.stack(pk)


def abc_mask3(n, n_abc, strength):
    """Absorbing mask of a 3-D grid: the 1-D mask of each axis multiplied together
    (ApplyABC multiplies the field by the mask, usefulsubs.py:584-609)."""
    m = [abc_mask(nn, na, strength) for nn, na in zip(n, n_abc)]
    return m[0][:, None, None] * m[1][None, :, None] * m[2][None, None, :]


class Pstd3D:
    """Field state E = (Ex, Ey, Ez), H = (Hx, Hy, Hz), each (3, nx, ny, nz) complex.
    Leapfrog of the curl equations with spectral derivatives (the q-space derivative
    f (i q) of usefulsubs.py:233-380 along each axis): H^{n+1/2} = H^{n-1/2} - dt/mu0
    curl E^n, E^{n+1} = mask (E^n + dt/eps (curl H^{n+1/2} - J))."""

    def __init__(self, n, d, epsr, n_abc=(0, 0, 0), strength=0.0):
        self.n, self.d, self.epsr = tuple(n), tuple(d), epsr
        grids = [pstd_grid(nn, dd) for nn, dd in zip(n, d)]
        self.x = [g[0] for g in grids]
        self.q = [g[1] for g in grids]
        self.mask = abc_mask3(n, n_abc, strength)
        self.masked = any(a > 0 for a in n_abc)
        self.Q = np.meshgrid(*self.q, indexing="ij")

    def curl(self, F):
        fk = [np.fft.fftn(F[c]) for c in range(3)]
        qx, qy, qz = self.Q
        ck = [1j * (qy * fk[2] - qz * fk[1]), 1j * (qz * fk[0] - qx * fk[2]),
              1j * (qx * fk[1] - qy * fk[0])]
        return np.stack([np.fft.ifftn(c) for c in ck])

    def update_h(self, E, H, dt):
        H = H - (dt / MU0) * self.curl(E)
        return H * self.mask if self.masked else H

    def update_e(self, E, H, J, dt):
        ie = dt / (EPS0 * self.epsr)
        E = E + ie * self.curl(H)
        if J is not None:
            E = E - ie * J
        return E * self.mask if self.masked else E

    def step(self, E, H, J, dt):
        H = self.update_h(E, H, dt)
        return self.update_e(E, H, J, dt), H

    def energy(self, E, H_prev, H_next):
        e = EPS0 * self.epsr * np.sum(np.abs(E) ** 2)
        h = MU0 * np.sum(np.real(H_prev * np.conj(H_next)))
        return e + h


class CoupledGrid3:
    """Wires along the z axis of a 3-D grid (one oracle ``Wire`` per wire, its 1-based
    index and (x, y) position), centred at z = 0: the wire's (x, y, z) components are
    the grid's (z, x, y).  Field -> wire: bilinear in x, y on every grid z, the spline
    along z evaluated at the wire's r (Prop2QW, qwoptics.py:667-715); wire -> grid:
    each source's spline evaluated at the grid z, gated by exp(-d^2 / (2 a^2)) in x and
    y (the SHO gates of rhoPJ.py:383-389 with QWPlacement, :655-702) around the wire;
    J = (P^{n+1} - P^n)/dt plus a current sheet in the plane x = x[src_index] along
    component pol with the profile exp(-(y^2 + z^2)/waist^2)."""

    def __init__(self, pstd, wires, windex, wxy, gate, src_index=-1, pol=1, E0=0.0, tau=1.0,
                 w0=0.0, tpeak=0.0, t0=0.0, waist=0.0):
        self.p = pstd
        self.wires, self.windex = wires, list(windex)
        self.wxy = np.asarray(wxy, float).reshape(-1, 2)
        self.gate = gate
        self.src_index, self.pol, self.E0, self.tau, self.w0 = src_index, pol, E0, tau, w0
        self.tpeak, self.t0, self.waist = tpeak, t0, waist
        self.eta = np.sqrt(MU0 / (EPS0 * pstd.epsr))
        self.Pold = np.zeros((3,) + pstd.n, complex)
        self.n = 0

    def _cell(self, g, v):
        i = int(np.searchsorted(g, v, side="right") - 1)
        i = min(max(i, 0), len(g) - 2)
        return i, (v - g[i]) / (g[i + 1] - g[i])

    def lines(self, E):
        """Grid fields on the line of every wire: [w][f][k], f the wire's component."""
        xg, yg = self.p.x[0], self.p.x[1]
        out = []
        for xw, yw in self.wxy:
            i0, fx = self._cell(xg, xw)
            j0, fy = self._cell(yg, yw)
            w00, w10 = (1 - fx) * (1 - fy), fx * (1 - fy)
            w01, w11 = (1 - fx) * fy, fx * fy
            fl = []
            for src in (2, 0, 1):
                F = E[src]
                fl.append(w00 * F[i0, j0] + w10 * F[i0 + 1, j0] + w01 * F[i0, j0 + 1] +
                          w11 * F[i0 + 1, j0 + 1])
            out.append(fl)
        return out

    def sample(self, E):
        zg = self.p.x[2]
        out = []
        for wi, fl in zip(self.wires, self.lines(E)):
            ek = []
            for f in fl:
                b, c, d = O.spline_coeffs(zg, f)
                v = rescale_vec(zg, b, c, d, f, wi.g["r"]) * wi.window
                ek.append(O.fftg(np.real(v).astype(complex)))
            out.append(ek)
        return out

    def deposit(self, srcs):
        """srcs: per wire real-space (Px, Py, Pz, re, rh).  Returns (Pg (3, ...), rho)."""
        xg, yg, zg = self.p.x
        Pg = np.zeros((3,) + self.p.n, complex)
        rho = np.zeros(self.p.n, complex)
        a2 = 2.0 * self.gate ** 2
        for wi, (xw, yw), s in zip(self.wires, self.wxy, srcs):
            r = wi.g["r"]
            vals = []
            for comp in s:
                b, c, d = O.spline_coeffs(r, comp)
                vals.append(rescale_vec(r, b, c, d, comp, zg))
            dl = [vals[1], vals[2], vals[0], vals[4] - vals[3]]
            g = np.exp(-(xg - xw) ** 2 / a2)[:, None] * np.exp(-(yg - yw) ** 2 / a2)[None, :]
            for c in range(3):
                Pg[c] += g[:, :, None] * dl[c][None, None, :]
            rho += g[:, :, None] * dl[3][None, None, :]
        return Pg, rho

    def current(self, Pg, dt):
        J = (Pg - self.Pold) / dt
        if self.src_index >= 0:
            th = self.t0 + (self.n + 0.5) * dt
            a = (th - self.tpeak) / self.tau
            einc = np.exp(-a * a) * np.cos(self.w0 * (th - self.tpeak))
            jamp = -2.0 * self.E0 / (self.eta * self.p.d[0])
            yg, zg = self.p.x[1], self.p.x[2]
            prof = np.ones((len(yg), len(zg)))
            if self.waist > 0:
                prof = np.exp(-(yg[:, None] ** 2 + zg[None, :] ** 2) / self.waist ** 2)
            J[self.pol, self.src_index] += jamp * einc * prof
        self.Pold = Pg.copy()
        return J

    def step(self, states, E, H, dt):
        """states: per wire [P, C, D] (updated in place).  Returns (E, H, srcs)."""
        eks = self.sample(E)
        H = self.p.update_h(E, H, dt)
        srcs = []
        for i, (wi, st) in enumerate(zip(self.wires, states)):
            z = [np.zeros_like(eks[i][0])] * 3
            P, C, D, Px, Py, Pz, re, rh = wi.rk4_step(st[0], st[1], st[2], eks[i], z, dt,
                                                     self.windex[i])
            st[0], st[1], st[2] = P, C, D
            srcs.append([O.ifftg(a) for a in (Px, Py, Pz, re, rh)])
        Pg, rho = self.deposit(srcs)
        J = self.current(Pg, dt)
        E = self.p.update_e(E, H, J, dt)
        self.n += 1
        return E, H, srcs
