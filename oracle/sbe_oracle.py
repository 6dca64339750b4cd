"""CPU FP64 restatement of the PulseSuite quantum-wire SBE path (the oracle).

TEST INFRASTRUCTURE ONLY.  This module is imported by ``tests/``, by
``__graft_entry__.smoke()`` (to check the CUDA path) and by ``bench.py``'s CPU baseline
and reference arm; nothing in ``pulsesuite_gb300`` imports or calls it.

Every function restates, in vectorised NumPy, the arithmetic of one function of
the reference (rahulranjansah/pulsesuite, ``src/pulsesuite/...``) and cites the
file:line it follows.  Reference quirks are kept as written (not fixed); each is
noted where it appears.  The oracle is pinned to the reference by the golden
vectors in ``tests/golden`` (made by ``tests/golden/make_golden.py`` from the
reference's own functions).
"""

import math

import numpy as np

# CODATA values used by the reference through scipy.constants (scipy 1.18).
HBAR = 1.0545718176461565e-34
E0 = 1.602176634e-19
EPS0 = 8.8541878188e-12
ME0 = 9.1093837139e-31
KB = 1.380649e-23
C0 = 299792458.0
PI = np.pi
TWOPI = 2.0 * np.pi
EULER = 0.5772156649015329
SMALL = 1e-200          # SBEs.py:4705 (SBESolver.small)
QW_SMALL = 1e-100       # qwoptics.py:598 (QWOptics._small)

# ----------------------------------------------------------------------------
# FFT with the reference's normalisation
# ----------------------------------------------------------------------------


def fftg(f):
    """usefulsubs.py:2245-2268  FFTG: F = -fft(F)/N."""
    f = np.asarray(f, dtype=complex)
    return -np.fft.fft(f) / len(f)


def ifftg(f):
    """usefulsubs.py:2271-2293  iFFTG: F = -ifft(F)*N."""
    f = np.asarray(f, dtype=complex)
    return -np.fft.ifft(f) * len(f)


# ----------------------------------------------------------------------------
# Grid and derived wire constants
# ----------------------------------------------------------------------------


def space_array(n, length):
    """typespace.py:815-849  GetSpaceArray: linspace(-L/2, L/2, N)."""
    if n == 1:
        return np.array([0.0])
    return np.linspace(-length / 2.0, length / 2.0, n)


def k_array(n, length):
    """typespace.py:852-886  GetKArray: centred k grid with dk = 2pi/L."""
    if n == 1:
        return np.array([0.0])
    dk = TWOPI / length if length > 0 else 1.0
    k = np.arange(n, dtype=float) * dk
    return k - k[n // 2]


def array0_index(x):
    """usefulsubs.py:1012-1035  GetArray0Index."""
    dx = x[2] - x[1]
    xi = np.round((x + 0.1 * dx) / dx).astype(np.int32)
    for i in range(len(x)):
        if xi[i] == 0:
            return i
    return None


def wire_grid(nk, L):
    """SBEs.py:4754-4760, 5028-5040, 5042-5051 with an explicit (Nk, L).

    Nr = 2*Nk + 2 (the reference computes Nk_odd, Nr = 2*Nk_odd, Nk = Nk_odd-1).
    kr[k] = dkr*(-dnk + k - 0.5); r spans [-L, L]; Qr is FFT ordered; kkp[k,kp] =
    round((kr[k]-kr[kp])/dkr) + NQ0.
    """
    dkr = TWOPI / (2.0 * L)
    nr = 2 * nk + 2
    dnk = (nk - 1) // 2
    kr = np.array([dkr * (-dnk + k - 0.5) for k in range(nk)])
    r = space_array(nr, 2 * L)
    Qr = k_array(nr, 2 * L)
    Qr = np.roll(Qr, nr // 2)
    Qr[0] = -Qr[0]
    NQ0 = array0_index(Qr)
    kkp = np.round((kr[:, None] - kr[None, :]) / dkr).astype(np.int64) + NQ0
    dr = (r[2] - r[1]) * (nr - 1) / float(nr)
    return dict(nk=nk, nr=nr, dkr=dkr, L=L, kr=kr, r=r, Qr=Qr, NQ0=NQ0, kkp=kkp, dr=dr,
                NK0=dnk + 1)


def grid_from_params(L, gap, me):
    """SBEs.py:4754-4758: Nk from L and the band gap (reference rule)."""
    kmax = np.sqrt(1.2 * gap * 2.0 * me / (HBAR ** 2))
    dkr = TWOPI / (2.0 * L)
    nk = int(np.floor(kmax / dkr) * 2 + 1) - 1
    return nk


def wire_constants(p, kr):
    """SBEs.py:4794-4823: dcv, alphae/h, ehint, area, qc, Ee, Eh (SI units).

    ``p`` holds SI values: gap (J), me, mh (kg), HO (J), Delta0 (m).
    """
    dcv = np.sqrt((E0 * HBAR) ** 2 / (6.0 * ME0 * p["gap"]) * (ME0 / p["me"] - 1.0))
    ae = np.sqrt(p["me"] * p["HO"]) / HBAR
    ah = np.sqrt(p["mh"] * p["HO"]) / HBAR
    ehint = np.sqrt(2.0 * ae * ah / (ae ** 2 + ah ** 2))
    qc = 2.0 * ae * ah / (ae + ah)
    area = np.sqrt(2.0 * PI) / np.sqrt(ae ** 2 + ah ** 2) * p["Delta0"]
    Ee = HBAR ** 2 * kr ** 2 / (2.0 * p["me"])
    Eh = HBAR ** 2 * kr ** 2 / (2.0 * p["mh"])
    return dict(dcv=dcv, alphae=ae, alphah=ah, ehint=ehint, qc=qc, area=area, Ee=Ee, Eh=Eh)


def yw(w):
    """qwoptics.py:1093-1106: (-1)**floor((w-1)/2)."""
    return (-1) ** int(np.floor((w - 1) / 2.0))


# ----------------------------------------------------------------------------
# Modified Bessel K0 (two variants, as in the reference)
# ----------------------------------------------------------------------------


def k0_truncated(x):
    """coulomb.py:39-66  _K03_jit, kept as written.

    x > 100 -> 0; x < 1e-10 -> 23; x < 2: -ln(x/2) - gamma plus the running
    term t_k = t_{k-1}*x^2/(4k^2) weighted by (1/k - gamma) (19 terms or until
    |t| < 1e-15); otherwise the leading asymptotic sqrt(pi/(2x)) e^-x.
    """
    x = float(x)
    if x > 100.0:
        return 0.0
    if x < 1e-10:
        return 23.0
    if x < 2.0:
        x2 = x * x
        res = -math.log(0.5 * x) - EULER
        term = 1.0
        for k in range(1, 20):
            term = term * 0.25 * x2 / (k * k)
            res = res + term * (1.0 / k - EULER)
            if abs(term) < 1e-15:
                break
        return res
    return math.sqrt(PI / (2.0 * x)) * math.exp(-x)


def k0_truncated_vec(x):
    """Array form of k0_truncated (same operations per element, with the series
    stopped per element at the first |term| < 1e-15 as the loop above does)."""
    x = np.asarray(x, dtype=float)
    out = np.where(x > 100.0, 0.0, 0.0)
    small = x < 1e-10
    ser = (x >= 1e-10) & (x < 2.0)
    asy = (x >= 2.0) & (x <= 100.0)
    xs = np.where(ser, x, 1.0)
    x2 = xs * xs
    res = -np.log(0.5 * xs) - EULER
    term = np.ones_like(xs)
    live = np.ones_like(xs, dtype=bool)
    for k in range(1, 20):
        term = np.where(live, term * 0.25 * x2 / (k * k), term)
        res = np.where(live, res + term * (1.0 / k - EULER), res)
        live = live & ~(np.abs(term) < 1e-15)
    xa = np.where(asy, x, 1.0)
    out = np.where(ser, res, out)
    out = np.where(asy, np.sqrt(PI / (2.0 * xa)) * np.exp(-xa), out)
    out = np.where(small, 23.0, out)
    return out


def _dfact2(n):
    r = 1.0
    while n > 1:
        r *= n
        n -= 2
    return r


# Asymptotic-series coefficients of Zhang & Jin's CIK01 (Computation of Special
# Functions, 1996): I0(z) ~ e^z/sqrt(2 pi z) sum a_k z^-k with
# a_k = ((2k-1)!!)^2/(k! 8^k), and I0(z)K0(z) ~ 1/(2z) sum b_k z^-2k with
# b_k = ((2k-1)!!)^3/((2k)!! 4^k).  Generated from the formulas.
_I0_ASY = [(_dfact2(2 * k - 1) ** 2) / (math.factorial(k) * 8.0 ** k) for k in range(1, 13)]
_K0I0_ASY = [(_dfact2(2 * k - 1) ** 3) / (_dfact2(2 * k) * 4.0 ** k) for k in range(1, 11)]


def _i0_cik(x):
    """usefulsubs.py:1700-1730 (real branch of cik01): I0 by series (x <= 18)
    or by the asymptotic series with 12/9/7 terms."""
    if x <= 18.0:
        s = 1.0
        cr = 1.0
        x2 = x * x
        for k in range(1, 51):
            cr = 0.25 * cr * x2 * (1.0 / (k * k))
            s = s + cr
            if abs(cr / s) < 1e-15:
                break
        return s
    k0 = 12 if x < 35.0 else (9 if x < 50.0 else 7)
    ca = math.exp(x) / math.sqrt(2.0 * PI * x)
    s = 1.0
    zr = 1.0 / x
    for k in range(1, k0 + 1):
        s = s + _I0_ASY[k - 1] * zr ** k
    return ca * s


def k0_cik(x):
    """usefulsubs.py:1649-1800  K03 -> cik01 real K0.

    x > 100 -> 0; x <= 9: K0 = -ln(x/2) - gamma + sum_k (x^2/4)^k/(k!)^2 (H_k + ct)
    until the relative change < 1e-15; x > 9: K0 = (1/(2x)) (1 + sum b_k x^-2k)/I0.
    The reference evaluates this in NumPy complex128 scalars, whose division
    multiplies by the reciprocal of the divisor; the series below does the same
    (the x <= 9 sum cancels to ~1e-8 of its terms, so the rounding shows).
    """
    x = float(x)
    if x > 1e2:
        return 0.0
    if x == 0.0:
        return 1e30
    if x <= 9.0:
        cs = 0.0
        ct = -math.log(0.5 * x) - EULER
        w0 = 0.0
        cr = 1.0
        cw = 0.0
        x2 = x * x
        for k in range(1, 51):
            w0 = w0 + 1.0 / k
            cr = 0.25 * cr * (1.0 / (k * k)) * x2
            cs = cs + cr * (w0 + ct)
            if abs((cs - cw) / cs) < 1e-15:
                break
            cw = cs
        return ct + cs
    cb = 0.5 * (1.0 / x)
    zr2 = 1.0 / (x * x)
    s = 1.0
    for k in range(1, 11):
        s = s + _K0I0_ASY[k - 1] * zr2 ** k
    return cb * s * (1.0 / _i0_cik(x))


# ----------------------------------------------------------------------------
# Coulomb tables and screening (coulomb.py)
# ----------------------------------------------------------------------------


def vint(Q, y, a1, a2, Delta0):
    """coulomb.py:70-104, 113-176  Vint via _Vint_jit (uses the truncated K0).

    Sum over i, j in [Ny//4, 3Ny//4] of exp(-(a1 y_i)^2 - (a2 y_j)^2) *
    a1 a2/pi dy^2 * K0t(max(|Q|, (a1+a2)/4) * sqrt((y_i-y_j)^2 + Delta0^2)).
    """
    ny = len(y)
    n1, n2 = ny // 4, 3 * ny // 4
    yy = y[n1:n2 + 1]
    kmin = (a1 + a2) / 4.0
    dk = max(abs(Q), kmin)
    mult = a1 * a2 / PI * (y[1] - y[0]) ** 2
    rr = np.sqrt((yy[:, None] - yy[None, :]) ** 2 + Delta0 ** 2)
    ex = np.exp(-(a1 * yy[:, None]) ** 2 - (a2 * yy[None, :]) ** 2)
    k0 = k0_truncated_vec(dk * rr)
    return float(np.sum(ex * mult * k0))


def coulomb_tables(g, c, epsr, Delta0, me, mh):
    """coulomb.py:502-577 CalcCoulombArrays, 302-330 MakeQs, 580-630 CalcChi1D.

    Quirk kept: V0[k, q] is filled only where kkp[k, q] >= 0 (k >= q on the
    reference grid); the upper triangle stays zero.
    """
    nk, kr, kkp, Qr, r = g["nk"], g["kr"], g["kkp"], g["Qr"], g["r"]
    ae, ah = c["alphae"], c["alphah"]
    pref = E0 ** 2 / (TWOPI * EPS0 * epsr * g["L"])
    nq = len(Qr)
    need = np.unique(kkp[(kkp >= 0) & (kkp < nq)])
    tabs = {}
    fast = len(r) > 130
    if fast:
        # large grids: K0t depends on |i - j| only (up to the rounding of y_i - y_j),
        # so it is evaluated once per distance and gathered; the double sum itself
        # is kept as written
        ny = len(r)
        n1, n2 = ny // 4, 3 * ny // 4
        yy = r[n1:n2 + 1]
        idx = np.abs(np.arange(len(yy))[:, None] - np.arange(len(yy))[None, :])
        rdist = np.sqrt((yy - yy[0]) ** 2 + Delta0 ** 2)
    for name, (a1, a2) in (("eh", (ae, ah)), ("ee", (ae, ae)), ("hh", (ah, ah))):
        t = np.zeros(nq)
        if fast:
            ex = np.exp(-(a1 * yy[:, None]) ** 2 - (a2 * yy[None, :]) ** 2)
            mult = a1 * a2 / PI * (r[1] - r[0]) ** 2
            kmin = (a1 + a2) / 4.0
        for j in need:
            if fast:
                kd = k0_truncated_vec(max(abs(Qr[j]), kmin) * rdist)
                t[j] = pref * float(np.sum(ex * mult * kd[idx]))
            else:
                t[j] = pref * vint(Qr[j], r, a1, a2, Delta0)
        tabs[name] = t
    valid = (kkp >= 0) & (kkp < nq)
    idx = np.where(valid, kkp, 0)
    V0 = {n: np.where(valid, tabs[n][idx], 0.0) for n in tabs}
    qe = np.maximum(np.abs(kr[None, :] - kr[:, None]), ae / 2.0)
    qh = np.maximum(np.abs(kr[None, :] - kr[:, None]), ah / 2.0)
    Re = np.sqrt((2.0 / ae) ** 2 + Delta0 ** 2)
    Rh = np.sqrt((2.0 / ah) ** 2 + Delta0 ** 2)
    k0v = np.vectorize(k0_cik)
    scale = E0 ** 2 / (TWOPI * EPS0 * epsr * HBAR ** 2)
    chie = me * k0v(qe * Re) / qe * scale
    chih = mh * k0v(qh * Rh) / qh * scale
    return dict(Veh0=V0["eh"], Vee0=V0["ee"], Vhh0=V0["hh"], qe=qe, qh=qh,
                Chi1De=chie, Chi1Dh=chih, vq=tabs)


def screened_arrays(ct, screened, L, ne, nh):
    """coulomb.py:1172-1193 Eps1D, 1195-1230 CalcScreenedArrays.

    Quirk kept: eps = 1 - 2 Chi1De log|(qe - pi n)/(qe + n)| - (same for h),
    with n clamped to min(qe[1,1], qh[1,1])/pi*0.99.
    Returns VC (Nk, Nk, 3) and E1D (Nk, Nk).
    """
    nk = len(ne)
    VC = np.zeros((nk, nk, 3))
    VC[:, :, 0] = ct["Veh0"]
    VC[:, :, 1] = ct["Vee0"]
    VC[:, :, 2] = ct["Vhh0"]
    E1D = np.ones((nk, nk))
    if screened:
        n1d = np.sum(np.real(ne) + np.real(nh)) / 2.0 / L
        nmax = min(ct["qe"][1, 1], ct["qh"][1, 1]) / PI * 0.99
        n1d = min(n1d, nmax)
        E1D = (1.0 - ct["Chi1De"] * 2 * np.log(np.abs((ct["qe"] - PI * n1d) / (ct["qe"] + n1d)))
               - ct["Chi1Dh"] * 2 * np.log(np.abs((ct["qh"] - PI * n1d) / (ct["qh"] + n1d))))
        VC[:, :, 0] /= E1D
        VC[:, :, 1] /= E1D
        VC[:, :, 2] /= E1D
    return VC, E1D


# ----------------------------------------------------------------------------
# Phonons (phonons.py)
# ----------------------------------------------------------------------------


def fermi(En, temp):
    """phonons.py:317-340 FermiDistr (exp overflow -> 0 as in NumPy)."""
    with np.errstate(over="ignore"):
        return 1.0 / (np.exp(En / KB / temp) + 1.0)


def phonon_tables(Ee, Eh, epsr, Gph, Oph, temp, epsr0=10.0, epsrinf=8.2):
    """phonons.py:55-136 InitializePhonons (T, eps0/epsinf are module constants
    there: 77 K, 10, 8.2)."""
    N0 = 1.0 / (np.exp(HBAR * Oph / KB / temp) - 1.0)
    dE = Ee[None, :] * 0 + Ee[:, None] - Ee[None, :]      # [k, k1] = Ee[k]-Ee[k1]
    dH = Eh[:, None] - Eh[None, :]
    hO, hG = HBAR * Oph, HBAR * Gph
    EP = N0 / ((dE - hO) ** 2 + hG ** 2) + (N0 + 1.0) / ((dE + hO) ** 2 + hG ** 2)
    HP = N0 / ((dH - hO) ** 2 + hG ** 2) + (N0 + 1.0) / ((dH + hO) ** 2 + hG ** 2)
    idel = 1.0 - np.eye(len(Ee))
    EP = EP * 2.0 * Gph * idel
    HP = HP * 2.0 * Gph * idel
    Vscale = HBAR * Oph * epsr * (1.0 / epsrinf - 1.0 / epsr0)
    return dict(EP=EP, HP=HP, N0=N0, Vscale=Vscale)


def mbpe(ne, VC, E1D, pt):
    """phonons.py:140-201 MBPE: returns (Win_add, Wout_add).

    Quirk kept: Vep = VC[:,:,1]/E1D*Vscale with VC already screened.
    """
    Vep = VC[:, :, 1] / E1D * pt["Vscale"]
    EP = pt["EP"]
    win = (Vep * EP) @ ne
    wout = (Vep * EP.T) @ (1.0 - ne)
    return win, wout


def mbph(nh, VC, E1D, pt):
    """phonons.py:204-268 MBPH: returns (Win_add, Wout_add)."""
    Vhp = VC[:, :, 2] / E1D * pt["Vscale"]
    HP = pt["HP"]
    win = (Vhp.T * HP) @ nh
    wout = (Vhp * HP).T @ (1.0 - nh)
    return win, wout


# ----------------------------------------------------------------------------
# Dephasing (dephasing.py)
# ----------------------------------------------------------------------------


def dephasing_tables(ky, me, mh):
    """dephasing.py:472-535 InitializeDephasing: index maps and xe, xh."""
    nk = len(ky)
    dk = ky[1] - ky[0] if nk > 1 else 1.0
    kmax = ky[nk - 1] + dk
    kmin = ky[0] - dk
    nk0 = (nk - 1) // 2 + 1

    def idx(v):
        return (np.round(np.clip(v, kmin, kmax) / dk)).astype(np.int64) + nk0 - 1

    K = ky[:, None]
    Q = ky[None, :]
    k_p_q = idx(K + Q)
    k_m_q = idx(K - Q)
    k1p0 = ((me + mh) * Q - 2 * mh * K) / 2.0 / me
    k1p = idx(k1p0)
    k1p_m_q = idx(k1p0 - Q)
    k10 = ((me + mh) * Q - 2 * me * K) / 2.0 / mh
    k1 = idx(k10)
    k1_m_q = idx(k10 - Q)
    xe = me / HBAR ** 2 * np.abs(ky) / (np.abs(ky) + dk * 1e-5) ** 2 / dk
    xh = mh / HBAR ** 2 * np.abs(ky) / (np.abs(ky) + dk * 1e-5) ** 2 / dk
    return dict(k_p_q=k_p_q, k_m_q=k_m_q, k1p=k1p, k1p_m_q=k1p_m_q, k1=k1, k1_m_q=k1_m_q,
                xe=xe, xh=xh)


def vxx2(q, V):
    """dephasing.py:362-378 Vxx2: V[round(|q/dq|), 0]**2 (round half to even)."""
    dq = q[1] - q[0] if len(q) > 1 else 1.0
    iq = np.round(np.abs(q / dq)).astype(np.int32)
    return V[iq, 0] ** 2


def _gather(arr_ext, idx, n):
    """Gather from a zero-padded (n+2) array at idx+1 with the kernel's
    validity test 1 <= idx+1 < n+1."""
    ok = (idx + 1 >= 1) & (idx + 1 < n + 1)
    return np.where(ok, arr_ext[np.clip(idx + 1, 0, n + 1)], 0.0), ok


def gamma_e(ky, ne0, nh0, VC, dt_):
    """dephasing.py:29-63 _CalcGammaE_jit, 541-581 CalcGammaE."""
    nk = len(ky)
    Veh2 = vxx2(ky, VC[:, :, 0])
    Vee2 = vxx2(ky, VC[:, :, 1])
    ne = np.zeros(nk + 2)
    nh = np.zeros(nk + 2)
    ne[1:nk + 1] = np.real(ne0)
    nh[1:nk + 1] = np.real(nh0)
    se = np.zeros(nk + 2)
    sh = np.zeros(nk + 2)
    se[1:nk + 1] = 1.0 - ne[1:nk + 1]
    sh[1:nk + 1] = 1.0 - nh[1:nk + 1]
    a, ok = _gather(ne, dt_["k_p_q"], nk)
    b, _ = _gather(se, dt_["k_p_q"], nk)
    term_ee = np.where(ok, PI / HBAR * Vee2[None, :] * a * b * np.abs(dt_["xe"])[None, :], 0.0)
    n1, ok1 = _gather(nh, dt_["k1p_m_q"], nk)
    s1, _ = _gather(sh, dt_["k1p_m_q"], nk)
    n2, ok2 = _gather(nh, dt_["k1p"], nk)
    s2, _ = _gather(sh, dt_["k1p"], nk)
    n3, ok3 = _gather(ne, dt_["k_m_q"], nk)
    s3, _ = _gather(se, dt_["k_m_q"], nk)
    okeh = ok1 & ok2 & ok3
    term_eh = np.where(okeh, PI / HBAR * Veh2[None, :] * (n1 * s2 * n3 + s1 * n2 * s3)
                       * np.abs(dt_["xh"])[None, :], 0.0)
    return term_ee.sum(axis=1) + term_eh.sum(axis=1)


def gamma_h(ky, ne0, nh0, VC, dt_):
    """dephasing.py:66-100 _CalcGammaH_jit, 584-625 CalcGammaH."""
    nk = len(ky)
    Veh2 = vxx2(ky, VC[:, :, 0])
    Vhh2 = vxx2(ky, VC[:, :, 2])
    ne = np.zeros(nk + 2)
    nh = np.zeros(nk + 2)
    ne[1:nk + 1] = np.real(ne0)
    nh[1:nk + 1] = np.real(nh0)
    se = np.zeros(nk + 2)
    sh = np.zeros(nk + 2)
    se[1:nk + 1] = 1.0 - ne[1:nk + 1]
    sh[1:nk + 1] = 1.0 - nh[1:nk + 1]
    a, ok = _gather(nh, dt_["k_p_q"], nk)
    b, _ = _gather(sh, dt_["k_p_q"], nk)
    term_hh = np.where(ok, PI / HBAR * Vhh2[None, :] * a * b * np.abs(dt_["xh"])[None, :], 0.0)
    n1, ok1 = _gather(ne, dt_["k1_m_q"], nk)
    s1, _ = _gather(se, dt_["k1_m_q"], nk)
    n2, ok2 = _gather(ne, dt_["k1"], nk)
    s2, _ = _gather(se, dt_["k1"], nk)
    n3, ok3 = _gather(nh, dt_["k_m_q"], nk)
    s3, _ = _gather(sh, dt_["k_m_q"], nk)
    okeh = ok1 & ok2 & ok3
    term_eh = np.where(okeh, PI / HBAR * Veh2[None, :] * (n1 * s2 * n3 + s1 * n2 * s3)
                       * np.abs(dt_["xe"])[None, :], 0.0)
    return term_hh.sum(axis=1) + term_eh.sum(axis=1)


def _lrtz(a, b):
    """dephasing.py:221-224 Lrtz: (b/pi)/(a^2+b^2)."""
    return (b / PI) / (a ** 2 + b ** 2)


def _vsq(VC, nk):
    """dephasing.py:381-414: Vsq[q+Nk] = VC[|q|,0,:]**2 for 1 <= |q| < Nk."""
    vsq = np.zeros((2 * nk + 1, 3))
    for q in range(1, nk):
        vsq[q + nk, :] = VC[q, 0, :] ** 2
        vsq[-q + nk, :] = VC[q, 0, :] ** 2
    return vsq


def _offdiag_D(n_a, n_b, Ea, Eb, vsq_aa, vsq_ab, gaa, gab):
    """dephasing.py:227-270 (_CalcOffDiagDeph_E2_jit) and 273-317 (_H2_jit).

    ``a`` is the carrier whose matrix is built, ``b`` the other species.
    Quirk kept: in the a-a sum q runs to p-1, so p-q = 0 is skipped.
    """
    nk = len(n_a)
    D = np.zeros((2 * nk + 1, nk))
    ks = np.arange(nk)
    for q in range(-nk, nk + 1):
        kk = ks[(ks + q >= 0) & (ks + q < nk)]
        if kk.size == 0:
            continue
        # a-a part: p in [max(q+1, 0), min(q+nk-1, nk-1)]
        plo, phi = max(q + 1, 0), min(q + nk - 1, nk - 1)
        if plo <= phi and vsq_aa[q + nk] != 0.0:
            pp = np.arange(plo, phi + 1)
            K = kk[:, None]
            P = pp[None, :]
            Ed = Ea[K + q] + Ea[P - q] - Ea[P] - Ea[K]
            occ = (n_a[P - q] * (1.0 - n_a[P]) * (1.0 - n_a[K])
                   + (1.0 - n_a[P - q]) * n_a[P] * n_a[K])
            D[q + nk, kk] += (vsq_aa[q + nk] * _lrtz(Ed, HBAR * gaa) * occ).sum(axis=1)
        # a-b part: p in [max(0, -q), min(nk-1, nk-1-q)]
        plo, phi = max(0, -q), min(nk - 1, nk - 1 - q)
        if plo <= phi and vsq_ab[q + nk] != 0.0:
            pp = np.arange(plo, phi + 1)
            K = kk[:, None]
            P = pp[None, :]
            Ed = Ea[K + q] + Eb[P + q] - Eb[P] - Ea[K]
            occ = (n_b[P + q] * (1.0 - n_b[P]) * (1.0 - n_a[K])
                   + (1.0 - n_b[P + q]) * n_b[P] * n_a[K])
            D[q + nk, kk] += (vsq_ab[q + nk] * _lrtz(Ed, HBAR * gab) * occ).sum(axis=1)
    return D * PI / HBAR


def offdiag_De(ne, nh, Ee, Eh, gee, geh, VC):
    """dephasing.py:381-396 CalcOffDiagDeph_E2 (occupations enter as |n|)."""
    nk = len(ne)
    vsq = _vsq(VC, nk)
    return _offdiag_D(np.abs(ne), np.abs(nh), Ee, Eh, vsq[:, 1], vsq[:, 0], gee, geh)


def offdiag_Dh(ne, nh, Ee, Eh, ghh, geh, VC):
    """dephasing.py:399-414 CalcOffDiagDeph_H2."""
    nk = len(ne)
    vsq = _vsq(VC, nk)
    return _offdiag_D(np.abs(nh), np.abs(ne), Eh, Ee, vsq[:, 2], vsq[:, 0], ghh, geh)


def offdiag_contract(Dh, De, p):
    """dephasing.py:320-356 _OffDiagDephasing2_jit in matrix form.

    x = i hbar (A @ p + p @ B.T), A[kh, j] = Dh[j-kh+Nk, kh], B[ke, j] =
    De[j-ke+Nk, ke], with the q = 0 (diagonal) entries removed by undel.
    """
    nk = p.shape[0]
    j = np.arange(nk)
    qi = j[None, :] - j[:, None] + nk          # [row, j] -> q index
    A = Dh[qi, j[:, None]]
    B = De[qi, j[:, None]]
    np.fill_diagonal(A, 0.0)
    np.fill_diagonal(B, 0.0)
    return 1j * HBAR * (A @ p + p @ B.T)


def offdiag_dephasing2(ne, nh, p, Ee, Eh, g, VC):
    """dephasing.py:714-743 OffDiagDephasing2 (g = [gam_eh, gam_e, gam_h]).

    Quirk kept: De uses (g[0], g[2]) and Dh uses (g[1], g[2]).
    """
    De = offdiag_De(ne, nh, Ee, Eh, g[0], g[2], VC)
    Dh = offdiag_Dh(ne, nh, Ee, Eh, g[1], g[2], VC)
    return offdiag_contract(Dh, De, p), De, Dh


# ----------------------------------------------------------------------------
# Hamiltonians and the SBE right-hand side (SBEs.py)
# ----------------------------------------------------------------------------


def calc_h(Meh, Wee, Whh, C, D, p, VC, Ee, Eh, gap, excitons, lf, freepot):
    """SBEs.py:1044-1131 _CalcH_fallback (vectorised per momentum shift q)."""
    nk = p.shape[0]
    V = np.zeros((2 * nk + 1, 3))
    for q in range(1, nk):
        V[nk + q, :] = VC[q, 0, :]
        V[nk - q, :] = VC[q, 0, :]
    Heh = np.array(Meh, dtype=complex)
    Hee = np.zeros((nk, nk), complex)
    Hhh = np.zeros((nk, nk), complex)
    Hee[np.diag_indices(nk)] = Ee + gap
    Hhh[np.diag_indices(nk)] = Eh
    if freepot:
        Hee = Hee + Wee
        Hhh = Hhh + Whh
    pt, Ct, Dt = p.T, C.T, D.T
    if excitons:
        for q in range(-(nk - 1), nk):
            if q == 0:
                continue
            if q > 0:
                s, sq = slice(0, nk - q), slice(q, nk)
            else:
                s, sq = slice(-q, nk), slice(0, nk + q)
            Heh[s, s] += V[nk + q, 0] * pt[sq, sq]
            if lf:
                Hee[s, s] -= V[nk + q, 1] * Ct[sq, sq]
                Hhh[s, s] -= V[nk + q, 2] * Dt[sq, sq]
        if lf:
            for d in range(-(nk - 1), nk):
                if d == 0:
                    continue
                trC = np.trace(C, offset=d)
                trDm = np.trace(D, offset=-d)
                trD = np.trace(D, offset=d)
                trCm = np.trace(C, offset=-d)
                vee = V[nk + d, 1] * trC - V[nk + d, 0] * trDm
                vhh = V[nk + d, 2] * trD - V[nk + d, 0] * trCm
                if d > 0:
                    k2 = np.arange(0, nk - d)
                    k1 = k2 + d
                else:
                    k1 = np.arange(0, nk + d)
                    k2 = k1 - d
                Hee[k1, k2] += vee
                Hhh[k1, k2] += vhh
        else:
            cd = np.diag(C)
            dd = np.diag(D)
            j = np.arange(nk)
            for k in range(nk):
                m = j != k
                Hee[k, k] -= np.sum(V[nk + (j[m] - k), 1] * cd[m])
                Hhh[k, k] -= np.sum(V[nk + (j[m] - k), 2] * dd[m])
    return Heh, Hee, Hhh


def calc_meh(Ex, Ey, Ez, w, kkp, ehint, dcv):
    """SBEs.py:5153-5163 _calc_Meh with qwoptics.py:618-622 dipoles.

    Meh[ke,kh] = -ehint (Xcv Ex[kkp] + Ycv Ey[kkp] yw(w) + Zcv Ez[kkp] (-1)^w),
    Xcv[ke,kh] = dcv (-1)^kh, Ycv = dcv, Zcv = -dcv; negative kkp wraps (FFT order).
    """
    nk = kkp.shape[0]
    sgn = (-1.0) ** np.arange(nk)
    Xcv = dcv * np.broadcast_to(sgn[None, :], (nk, nk))
    return (-ehint * Xcv * Ex[kkp] - ehint * dcv * Ey[kkp] * yw(w)
            - ehint * (-dcv) * Ez[kkp] * (-1) ** w)


def dpdt(C, D, p, Heh, Hee, Hhh, GamE, GamH, OffP):
    """SBEs.py:2189-2207 _dpdt_fallback in matrix form (p stored [kh, ke])."""
    r = (Hhh @ p + p @ Hee.T - Heh.T @ C - (Heh @ D).T + Heh.T
         - 1j * HBAR * (GamE[None, :] + GamH[:, None]) * p + OffP)
    return r / (1j * HBAR)


def dCdt(C, D, p, Heh, Hee, Hhh, GamE, GamH, OffE):
    """SBEs.py:2481-2499 _dCdt_fallback in matrix form."""
    r = C @ Hee.T - Hee.T @ C + p.conj().T @ Heh.T - Heh.conj() @ p
    return r / (1j * HBAR)


def dDdt(C, D, p, Heh, Hee, Hhh, GamE, GamH, OffH):
    """SBEs.py:2779-2797 _dDdt_fallback in matrix form."""
    r = D @ Hhh.T - Hhh.T @ D + p.conj() @ Heh - Heh.conj().T @ p.T
    return r / (1j * HBAR)


# ----------------------------------------------------------------------------
# Optics: window, e^{ikr}, sources, field resampling (qwoptics.py)
# ----------------------------------------------------------------------------


def qw_window(r, L):
    """qwoptics.py:628-648 CalcQWWindow: exp(-(r/(L/2))**150)."""
    return np.exp(-((r / (L / 2.0)) ** 150))


def expikr(kr, r):
    """qwoptics.py:652-663 CalcExpikr: exp(i k r), shape (Nk, Nr)."""
    return np.exp(1j * np.outer(kr, r))


def qw_polarization3(r, kr, p, ehint, area, L, w, dcv, window, E):
    """qwoptics.py:50-76 and 809-940 QWPolarization3 (matrix form).

    Px[r] = win Re(sum_{ke,kh} p[kh,ke] Xvc0[kh,ke] e^{i ke r} e^{-i kh r}),
    Xvc0 = conj(Xcv0.T); then x 2 ehint/(area L) and FFTG.
    """
    nk = len(kr)
    sgn = (-1.0) ** np.arange(nk)
    Xvc0 = np.conj((dcv * np.broadcast_to(sgn[None, :], (nk, nk))).T)
    Yvc0 = np.conj(np.full((nk, nk), dcv, dtype=complex).T)
    Zvc0 = np.conj(np.full((nk, nk), -dcv, dtype=complex).T)
    Ec = np.conj(E)
    out = []
    for M, f in ((Xvc0, 1.0), (Yvc0, float(yw(w))), (Zvc0, float((-1) ** w))):
        G = (p * M) @ E
        s = np.real(np.sum(G * Ec, axis=0)) * window * f
        out.append(fftg(s * 2 * ehint / area / L))
    return out


def qw_rho5(r, L, C, D, ne, nh, window, E):
    """qwoptics.py:361-374 and 942-1071 QWRho5 (matrix form).

    re[r] = sum C[k1,k2] e^{-i k1 r} e^{i k2 r} win/(2L); rh with conj(D);
    boundary-mean subtraction, renormalisation to sum|n|, FFTG.
    """
    nr = len(r)
    dr = r[1] - r[0]
    NeT = np.sum(np.abs(ne)) + 1e-50
    NhT = np.sum(np.abs(nh)) + 1e-50
    Ec = np.conj(E)
    re = np.sum(Ec * (C @ E), axis=0) * window / (2.0 * L)
    rh = np.sum(Ec * (np.conj(D) @ E), axis=0) * window / (2.0 * L)
    re = re - np.real(np.sum(re[0:10]) + np.sum(re[nr - 10:nr])) / 20.0
    rh = rh - np.real(np.sum(rh[0:10]) + np.sum(rh[nr - 10:nr])) / 20.0
    re = re * NeT / (np.sum(np.abs(re)) * dr + QW_SMALL)
    rh = rh * NhT / (np.sum(np.abs(rh)) * dr + QW_SMALL)
    return fftg(re), fftg(rh)


def spline_coeffs(x, y):
    """spliner.py:1329-1394 spline_dpc (Forsythe-Malcolm-Moler cubic spline)."""
    n = len(x)
    y = np.asarray(y, dtype=complex)
    b = np.zeros(n, complex)
    c = np.zeros(n, complex)
    d = np.zeros(n, complex)
    if n < 3:
        b[0] = (y[1] - y[0]) / (x[1] - x[0])
        b[1] = b[0]
        return b, c, d
    d[0] = x[1] - x[0]
    c[1] = (y[1] - y[0]) / d[0]
    for i in range(1, n - 1):
        d[i] = x[i + 1] - x[i]
        b[i] = 2.0 * (d[i - 1] + d[i])
        c[i + 1] = (y[i + 1] - y[i]) / d[i]
        c[i] = c[i + 1] - c[i]
    b[0] = -d[0]
    b[n - 1] = -d[n - 2]
    c[0] = 0.0
    c[n - 1] = 0.0
    if n != 3:
        c[0] = c[2] / (x[3] - x[1]) - c[1] / (x[2] - x[0])
        c[n - 1] = c[n - 2] / (x[n - 1] - x[n - 3]) - c[n - 3] / (x[n - 2] - x[n - 4])
        c[0] = c[0] * d[0] ** 2 / (x[3] - x[0])
        c[n - 1] = -c[n - 1] * d[n - 2] ** 2 / (x[n - 1] - x[n - 4])
    for i in range(1, n):
        t = d[i - 1] / b[i - 1]
        b[i] = b[i] - t * d[i - 1]
        c[i] = c[i] - t * c[i - 1]
    c[n - 1] = c[n - 1] / b[n - 1]
    for i in range(n - 2, -1, -1):
        c[i] = (c[i] - d[i] * c[i + 1]) / b[i]
    b[n - 1] = (y[n - 1] - y[n - 2]) / d[n - 2] + d[n - 2] * (c[n - 2] + 2.0 * c[n - 1])
    for i in range(n - 1):
        b[i] = (y[i + 1] - y[i]) / d[i] - d[i] * (c[i + 1] + 2.0 * c[i])
        d[i] = (c[i + 1] - c[i]) / d[i]
        c[i] = 3.0 * c[i]
    c[n - 1] = 3.0 * c[n - 1]
    d[n - 1] = d[n - 2]
    return b, c, d


def locate(xx, x):
    """spliner.py:1137-1167 locate (binary search, clamped to [0, n-1])."""
    n = len(xx)
    if x < xx[0]:
        return 0
    if x >= xx[n - 1]:
        return n - 1
    jl, ju = 0, n
    while ju - jl > 1:
        jm = (ju + jl) // 2
        if x >= xx[jm]:
            jl = jm
        else:
            ju = jm
    return jl


def rescale_1d(x0, z0, x1):
    """spliner.py:153-189 rescale_1D_dpc: spline z0(x0) sampled at x1, 0 outside."""
    b, c, d = spline_coeffs(x0, z0)
    z0 = np.asarray(z0, dtype=complex)
    out = np.zeros(len(x1), complex)
    lo, hi = np.min(x0), np.max(x0)
    for i, u in enumerate(x1):
        if lo <= u <= hi:
            j = locate(x0, u)
            dx = u - x0[j]
            out[i] = z0[j] + dx * (b[j] + dx * (c[j] + dx * d[j]))
    return out


def prop2qw(RR, Exx, Eyy, Ezz, Vrr, r, window):
    """qwoptics.py:667-715 Prop2QW: spline to the wire grid, x window, real part, FFTG."""
    outs = []
    for f in (Exx, Eyy, Ezz, Vrr):
        v = rescale_1d(RR, f, r) * window
        outs.append(fftg(np.real(v).astype(complex)))
    return outs


def qw2prop(r, Px, Py, Pz, re, rh, RR, plasmonics):
    """qwoptics.py:717-805 QW2Prop: iFFTG, charge renormalisation, spline back."""
    dr = r[1] - r[0]
    dRR = RR[1] - RR[0]
    Px, Py, Pz, re, rh = (ifftg(a) for a in (Px, Py, Pz, re, rh))
    total = None
    if plasmonics:
        re = np.abs(re).astype(complex)
        rh = np.abs(rh).astype(complex)
        total = (np.sum(re) * dr + np.sum(rh) * dr + QW_SMALL) / 2.0
        re = re * total / (np.sum(re) * dr + QW_SMALL)
        rh = rh * total / (np.sum(rh) * dr + QW_SMALL)
    Pxx = rescale_1d(r, Px, RR)
    Pyy = rescale_1d(r, Py, RR)
    Pzz = rescale_1d(r, Pz, RR)
    RhoE = rescale_1d(r, re, RR)
    RhoH = rescale_1d(r, rh, RR)
    if plasmonics:
        RhoE = np.abs(RhoE).astype(complex)
        RhoH = np.abs(RhoH).astype(complex)
        RhoE = RhoE * total / (np.sum(RhoE) * dRR + QW_SMALL)
        RhoH = RhoH * total / (np.sum(RhoH) * dRR + QW_SMALL)
    return Pxx, Pyy, Pzz, RhoE, RhoH


# ----------------------------------------------------------------------------
# Relaxation and the reference leapfrog step (SBEs.py)
# ----------------------------------------------------------------------------


def mb_value(kind, a, b, d, Ee, Eh, ge, gh, lorentz):
    """coulomb.py:367-499 CalcMBArrays: the builder's value for 0-based (a, b, d).

    kind "eh": k30 = d + b - a, E = Ee[a] + Eh[b] - Eh[k30] - Ee[d], broadening
    geh = (ge + gh) / 2; "ee" / "hh": k30 = a + b - d with Ee (ge) / Eh (gh).
    UnDel[a+1, d+1] UnDel[b+1, k30+1] is (a != d) in both cases.  Zero where k30
    leaves [0, N).  Lorentzian 2 g / (E^2 + (hbar g)^2) or (2 pi / hbar) GaussDelta(E,
    hbar g) (coulomb.py:245-262).  a, b, d are integer arrays of one shape.
    """
    n = len(Ee)
    if kind == "eh":
        k30 = d + b - a
        g = (ge + gh) / 2.0
    else:
        k30 = a + b - d
        g = ge if kind == "ee" else gh
    ok = (k30 >= 0) & (k30 < n) & (a >= 0) & (b >= 0) & (d >= 0) & (a < n) & (b < n) & (d < n)
    aa, bb, dd, cc = [np.where(ok, x, 0) for x in (a, b, d, k30)]
    if kind == "eh":
        E = Ee[aa] + Eh[bb] - Eh[cc] - Ee[dd]
    elif kind == "ee":
        E = Ee[aa] + Ee[bb] - Ee[cc] - Ee[dd]
    else:
        E = Eh[aa] + Eh[bb] - Eh[cc] - Eh[dd]
    und = (aa != dd).astype(float)
    if lorentz:
        v = 2.0 * g * und * und / (E ** 2 + (HBAR * g) ** 2)
    else:
        hb = HBAR * g
        v = 2.0 * np.pi / HBAR * und * und * (1.0 / (np.sqrt(np.pi) * hb) * np.exp(-((E / hb) ** 2)))
    return np.where(ok, v, 0.0)


def _mb_store(kind, x, y, z, mb):
    """Table entry C[x, y, z] of the (N+1)^3 array as the scattering loops read it.

    Quirk kept (coulomb.py:957-1071): the loops index the 1-based table with
    k - 1, so storage index x holds the builder's 0-based x - 1 (0 for x = 0).
    """
    return mb_value(kind, x - 1, y - 1, z - 1, mb["Ee"], mb["Eh"], mb["ge"], mb["gh"],
                    mb["lorentz"]) * ((x >= 1) & (y >= 1) & (z >= 1))


def _vsq_full(VC, c):
    return VC[:, :, c] ** 2


def mbce(ne0, nh0, VC, mb):
    """coulomb.py:957-1011 _MBCE_core (via CoulombModule.MBCE, :1298-1311):
    returns (Win_add, Wout_add) of the electrons, Nk each."""
    n = len(ne0)
    ne = np.zeros(n + 1)
    nh = np.zeros(n + 1)
    ne[1:] = np.abs(np.real(ne0))
    nh[1:] = np.abs(np.real(nh0))
    Veh2 = _vsq_full(VC, 0)
    Vee2 = _vsq_full(VC, 1)
    q1, q2 = np.meshgrid(np.arange(1, n + 1), np.arange(1, n + 1), indexing="ij")
    win = np.zeros(n)
    wout = np.zeros(n)
    for k in range(1, n + 1):
        kp, k1 = q1, q2
        k1p = kp + k1 - k
        ok = (k1p >= 1) & (k1p <= n)
        k1pc = np.where(ok, k1p, 0)
        t1 = (Veh2[k - 1, k1 - 1] * (1.0 - nh[kp]) * nh[k1pc] * ne[k1]
              * _mb_store("eh", k - 1, kp - 1, k1 - 1, mb))
        s = np.sum(np.where(ok, t1, 0.0))
        k1p = kp + k - k1
        ok = (k1p >= 1) & (k1p <= n)
        k1pc = np.where(ok, k1p, 0)
        t2 = (Veh2[k1 - 1, k - 1] * (1.0 - ne[k1]) * (1.0 - nh[kp]) * nh[k1pc]
              * _mb_store("eh", k1 - 1, kp - 1, k - 1, mb))
        so = np.sum(np.where(ok, t2, 0.0))
        k2, k4 = q1, q2
        k30 = k + k2 - k4
        ok = (k30 >= 1) & (k30 <= n)
        k30c = np.where(ok, k30, 0)
        t3 = (Vee2[k - 1, k4 - 1] * (1.0 - ne[k2]) * ne[k30c] * ne[k4]
              * _mb_store("ee", k - 1, k2 - 1, k4 - 1, mb))
        s += np.sum(np.where(ok, t3, 0.0))
        k30 = k4 + k2 - k
        ok = (k30 >= 1) & (k30 <= n)
        k30c = np.where(ok, k30, 0)
        t4 = (Vee2[k4 - 1, k - 1] * (1.0 - ne[k4]) * (1.0 - ne[k2]) * ne[k30c]
              * _mb_store("ee", k4 - 1, k2 - 1, k - 1, mb))
        so += np.sum(np.where(ok, t4, 0.0))
        win[k - 1] = s
        wout[k - 1] = so
    return win, wout


def mbch(ne0, nh0, VC, mb):
    """coulomb.py:1014-1071 _MBCH_core (via CoulombModule.MBCH, :1313-1326):
    returns (Win_add, Wout_add) of the holes, Nk each."""
    n = len(ne0)
    ne = np.zeros(n + 1)
    nh = np.zeros(n + 1)
    ne[1:] = np.abs(np.real(ne0))
    nh[1:] = np.abs(np.real(nh0))
    Veh2 = _vsq_full(VC, 0)
    Vhh2 = _vsq_full(VC, 2)
    q1, q2 = np.meshgrid(np.arange(1, n + 1), np.arange(1, n + 1), indexing="ij")
    win = np.zeros(n)
    wout = np.zeros(n)
    for kp in range(1, n + 1):
        k, k1 = q1, q2
        k1p = kp + k1 - k
        ok = (k1p >= 1) & (k1p <= n)
        k1pc = np.where(ok, k1p, 0)
        t1 = (Veh2[k - 1, k1 - 1] * (1.0 - ne[k]) * nh[k1pc] * ne[k1]
              * _mb_store("eh", k - 1, kp - 1, k1 - 1, mb))
        s = np.sum(np.where(ok, t1, 0.0))
        k1p = kp + k - k1
        ok = (k1p >= 1) & (k1p <= n)
        k1pc = np.where(ok, k1p, 0)
        t2 = (Veh2[k1 - 1, k - 1] * (1.0 - ne[k]) * (1.0 - nh[k1pc]) * ne[k1]
              * _mb_store("eh", k - 1, k1pc - 1, k1 - 1, mb))
        so = np.sum(np.where(ok, t2, 0.0))
        k2p, k4p = q1, q2
        k3p = kp + k2p - k4p
        ok = (k3p >= 1) & (k3p <= n)
        k3pc = np.where(ok, k3p, 0)
        t3 = (Vhh2[kp - 1, k4p - 1] * (1.0 - nh[k2p]) * nh[k3pc] * nh[k4p]
              * _mb_store("hh", kp - 1, k2p - 1, k4p - 1, mb))
        s += np.sum(np.where(ok, t3, 0.0))
        k3p = k4p + k2p - kp
        ok = (k3p >= 1) & (k3p <= n)
        k3pc = np.where(ok, k3p, 0)
        t4 = (Vhh2[k4p - 1, kp - 1] * (1.0 - nh[k4p]) * (1.0 - nh[k2p]) * nh[k3pc]
              * _mb_store("hh", k4p - 1, k2p - 1, kp - 1, mb))
        so += np.sum(np.where(ok, t4, 0.0))
        win[kp - 1] = s
        wout[kp - 1] = so
    return win, wout


def dc_karray(nk, dky):
    """dcfield.py:39-58 GetKArray(Nk, (Nk - 1) dky) of DCFieldModule (:778)."""
    L = (nk - 1) * dky
    dk = 2.0 * PI / L if L > 0 else 1.0
    k = np.arange(nk, dtype=float) * dk
    return k - k[nk // 2]


def dc_transport(X, Edc, Eac, dt, dky, lf):
    """dcfield.py:1154-1236 ShiftN1D / ShiftN2D / Transport (DCTrans on): returns the
    shifted matrix (LF: the whole matrix; else the diagonal alone)."""
    dk = -E0 * (Edc + Eac) / HBAR * dt
    Y = dc_karray(X.shape[0], dky)
    if lf:
        F = np.fft.fft2(X)
        F = F * np.exp(-1j * (Y[:, None] + Y[None, :]) * dk)
        return np.fft.ifft2(F)
    d = np.fft.fft(np.diag(X).copy())
    d = d * np.exp(-1j * Y * dk)
    out = X.copy()
    np.fill_diagonal(out, np.fft.ifft(d))
    return out


def ek_renorm(n, En, V):
    """dcfield.py:339-344 _EkReNorm_jit: Ec(k) = En(k) + sum_k' n(k') (V[k,k] - V[k,k']) / 2."""
    return En + (np.diag(V) * np.sum(n) - V @ n) / 2.0


def drift_vt(n, Ec, dkk):
    """dcfield.py:348-359 _DriftVt_jit: centred dE/dk, linear ends, <dE/dk> / hbar."""
    nk = len(n)
    d = np.zeros(nk)
    d[1:nk - 1] = (Ec[2:] - Ec[:nk - 2]) / 2.0 / dkk
    d[0] = 2.0 * d[1] - d[2]
    d[nk - 1] = 2.0 * d[nk - 2] - d[nk - 3]
    return float(np.real(np.sum(d * n) / (1e-100 + np.sum(n)) / HBAR))


def wire_info(ne2, nh2, re, rh, Ek, src3, kr, me, mh, Ee, Eh, gap, L, dkr, VC):
    """The columns after the time of dataQW/info.WW.t.dat and dataQW/EP.WW.t.dat
    (SBEs.py:5769-5809): CalcVD (dcfield.py:128-151), densities, TotalEnergy and
    Temperature (usefulsubs.py:1185-1253, small = 1e-100), max |Re|, |Rh|, GetEDrift
    (the DC module's ERate: 0, SBEs never sets it), momenta, CalcI0 (dcfield.py:1110-1148
    with EkReNorm/DriftVt), CalcI0n (dcfield.py:103-125, complex); EP: the real parts
    of iFFTG(E)[Nr/2] and iFFTG(P)[Nr/2].  re, rh, the fields and the sources are the
    wire-k arrays the reference holds at that point."""
    def vd(m, n):
        return np.sum(np.real(n) * HBAR * kr / m) / np.sum(np.real(n) + 1e-200)

    def temp(n, E):
        return 2.0 * np.real(np.sum(n * E) / (np.sum(n) + 1e-100)) / KB

    def i0n(n, m):
        dk = kr[1] - kr[0] if len(kr) > 1 else 1.0
        return -E0 * np.sum(n * kr * HBAR / m) * 2.0 * dk

    ve = drift_vt(np.real(ne2), ek_renorm(np.real(ne2), Ee, VC[:, :, 1]), dkr)
    vh = drift_vt(np.real(nh2), ek_renorm(np.real(nh2), Eh, VC[:, :, 2]), dkr)
    i0 = np.real(-E0 * (ve + vh) * np.sum(ne2) * dkr * 2.0)
    info = [vd(me, ne2), vd(mh, nh2), np.real(2 * np.sum(ne2) / L), np.real(2 * np.sum(nh2) / L),
            np.real(np.sum(ne2 * (Ee + gap))) / E0, np.real(np.sum(nh2 * Eh)) / E0,
            temp(ne2, Ee), temp(nh2, Eh), np.max(np.abs(re)), np.max(np.abs(rh)), 0.0,
            np.real(HBAR * np.sum((ne2 - nh2) * kr)) * 2.0, np.real(HBAR * np.sum(ne2 * kr)),
            np.real(-HBAR * np.sum(nh2 * kr)), i0, i0n(ne2, me), i0n(1 - nh2, -mh)]
    nr = len(Ek[0])
    ep = [np.real(ifftg(E)[nr // 2]) for E in list(Ek) + list(src3)]
    return info, ep


def info_line(t, info):
    """One line of dataQW/info.WW.t.dat as SBEs.py:5772-5791 formats it (the two
    CalcI0n columns are complex and print as complex numbers)."""
    vals = [t] + list(info)
    return "".join(f"{v:18.6e} " for v in vals[:-1]) + f"{vals[-1]:18.6e}\n"


def ep_line(t, ep):
    """One line of dataQW/EP.WW.t.dat (SBEs.py:5800-5809)."""
    return " ".join(f"{v:18.6e}" for v in [t] + list(ep)) + "\n"


def calc_jfx(rho_new, rho_prev, dt, dx):
    """rhoPJ.py:491-515 CalcJfx."""
    d = (np.asarray(rho_new) - np.asarray(rho_prev)) / dt
    J = np.zeros(len(d), dtype=complex)
    for i in range(1, len(d)):
        J[i] = J[i - 1] - d[i] * dx
    return J


def qw_placement(fwire, gx, gy, gz):
    """rhoPJ.py:655-702 QWPlacement (returns the grid)."""
    g = (np.asarray(gx)[:, None, None] * np.asarray(gy)[None, :, None]) * np.asarray(gz)[None, None, :]
    return 0.0 + g * np.asarray(fwire)[:, None, None]


def locator(x, x0):
    """usefulsubs.py:1803-1830."""
    return max(0, min(int(np.searchsorted(x, x0, side="right")) - 1, len(x) - 2))


def e_at_xyz(f, x, y, z, x0, y0, z0):
    """usefulsubs.py:1996-2075 EAtXYZ (a singleton axis takes its one plane)."""
    idx, ws = [], []
    for a, a0 in ((x, x0), (y, y0), (z, z0)):
        if len(a) == 1:
            idx.append(0)
            ws.append((1.0, 0.0))
        else:
            i = locator(a, a0)
            al = (a0 - a[i]) / (a[i + 1] - a[i])
            idx.append(i)
            ws.append((1.0 - al, al))
    f0 = 0.0 + 0.0j
    for r in range(2):
        for q in range(2):
            for p in range(2):
                if (p and len(x) == 1) or (q and len(y) == 1) or (r and len(z) == 1):
                    continue
                f0 = f0 + ws[0][p] * ws[1][q] * ws[2][r] * f[idx[0] + p, idx[1] + q, idx[2] + r]
    return f0


EMISSION_TEMP = 77.0   # emission.py:28 _Temp: the module's own temperature, never set by SBEs.py


def emission_tables(dcv, epsr, geh, ehint, temp=EMISSION_TEMP):
    """emission.py:35-91 InitializeEmission with CalcHOmega (:220-255): the photon
    energy grid HOmega (midpoints, dhw) and the pre-calculated ``square`` array."""
    kBT = KB * temp
    hg = HBAR * geh
    hwmax = (kBT + hg) * 4.0
    dhw = min(kBT, hg) / 20.0
    nw = int(np.ceil(hwmax / dhw))
    if nw < 10:
        raise ValueError("temperature too low for the emission grid")
    how = np.array([0.0 + (n + 0.5) * dhw for n in range(nw)])
    lrtz = (hg / np.pi) / (how ** 2 + hg ** 2)
    square = (3.0 * dcv ** 2 * ehint / EPS0 / np.sqrt(epsr) * ehint / HBAR * lrtz
              * np.exp(-how / KB / temp))
    return dict(HOmega=how, square=square, dhw=how[1] - how[0])


def coulomb_ec(ne, nh, VC):
    """emission.py:133-171 Ec: Coulomb energy correction per k (ne, nh real)."""
    n = len(ne)
    Veh, Vee, Vhh = VC[:, :, 0], VC[:, :, 1], VC[:, :, 2]
    idel = 1.0 - np.eye(n)
    out = np.zeros(n)
    for k in range(n):
        out[k] = (np.sum(ne * (Vee[k, k] - Vee[:, k]) + nh * (Vhh[k, k] - Vhh[:, k]))
                  + np.sum(ne * Veh[k, k] * idel[:, k] - nh * Veh[k, k] * idel[:, k])
                  - Veh[k, k])
    return out


def spont_emission(ne, nh, Ee, Eh, gap, VC, et):
    """emission.py:94-131 SpontEmission with SpontIntegral (:174-198) and rho0
    (:201-217): Rsp per k."""
    Ek = gap + Ee + Eh + coulomb_ec(np.real(ne), np.real(nh), VC)
    how, sq = et["HOmega"], et["square"]
    rsp = np.zeros(len(ne))
    for k in range(len(ne)):
        hw = how + Ek[k]
        rsp[k] = np.sum(hw * (hw ** 2 / (C0 ** 3 * PI ** 2 * HBAR ** 3)) * sq) * et["dhw"]
    return rsp


def relax(ne, nh, VC, E1D, pt, dt, ehs, phonon, small=SMALL, mb=None, rsp=None):
    """SBEs.py:5228-5325 _relaxation with RelaxationE/H (SBEs.py:1709-1835): the
    carrier-carrier rates (EHs; ``mb`` = dict(Ee, Eh, ge, gh, lorentz)) first, then
    the phonon rates added; with ``rsp`` (Recomb) the spontaneous-emission decay
    after them (SBEs.py:5322-5325)."""
    if rsp is not None:
        ne, nh = relax(ne, nh, VC, E1D, pt, dt, ehs, phonon, small, mb)
        ne = ne * np.exp(-rsp * nh * dt)
        nh = nh * np.exp(-rsp * ne * dt)
        return ne, nh
    if not (phonon or ehs):
        return ne, nh
    n = len(ne)
    we_in, we_out, wh_in, wh_out = (np.zeros(n) for _ in range(4))
    if ehs:
        a, b = mbce(np.real(ne), np.real(nh), VC, mb)
        we_in, we_out = we_in + a, we_out + b
        a, b = mbch(np.real(ne), np.real(nh), VC, mb)
        wh_in, wh_out = wh_in + a, wh_out + b
    if phonon:
        a, b = mbpe(np.real(ne), VC, E1D, pt)
        we_in, we_out = we_in + a, we_out + b
        a, b = mbph(np.real(nh), VC, E1D, pt)
        wh_in, wh_out = wh_in + a, wh_out + b
    We = we_in + we_out
    Wh = wh_in + wh_out
    ne = np.exp(-We * dt) * ((-1 + np.exp(We * dt) + ne) * we_in + ne * we_out) / (We + small)
    nh = np.exp(-Wh * dt) * ((-1 + np.exp(Wh * dt) + nh) * wh_in + nh * wh_out) / (Wh + small)
    return ne, nh


FLAG_NAMES = ("Optics", "Excitons", "EHs", "Screened", "Phonon", "DCTrans", "LF",
              "FreePot", "DiagDph", "OffDiagDph", "Recomb")


class Wire:
    """All tables of one wire (SBEs.py:4623-4972 minus file output)."""

    def __init__(self, nk, L, params, flags, temp=77.0):
        p = dict(params)
        self.p = p
        self.flags = dict(flags)
        self.g = wire_grid(nk, L)
        self.c = wire_constants(p, self.g["kr"])
        self.temp = temp
        self.ct = coulomb_tables(self.g, self.c, p["epsr"], p["Delta0"], p["me"], p["mh"])
        self.pt = phonon_tables(self.c["Ee"], self.c["Eh"], p["epsr"], p["Gph"], p["Oph"], temp)
        # carrier-carrier scattering tables are evaluated on the fly (mb_value)
        self.mb = dict(Ee=self.c["Ee"], Eh=self.c["Eh"], ge=p["gam_e"], gh=p["gam_h"],
                       lorentz=bool(self.flags.get("LorentzDelta", False)))
        # SBEs.py:4905-4915: emission tables when Recomb is on
        self.et = (emission_tables(abs(self.c["dcv"]), p["epsr"], p["gam_eh"], self.c["ehint"])
                   if self.flags.get("Recomb", False) else None)
        self.dt = dephasing_tables(self.g["kr"], p["me"], p["mh"])
        self.window = qw_window(self.g["r"], L)
        self.E = expikr(self.g["kr"], self.g["r"])

    # preparation (SBEs.py:5173-5226)
    def prepare(self, p2, C2, D2, Ex, Ey, Ez, w):
        f, c, g, prm = self.flags, self.c, self.g, self.p
        nk = g["nk"]
        ne = np.diag(C2).copy()
        nh = np.diag(D2).copy()
        if f["Optics"]:
            Meh = calc_meh(Ex, Ey, Ez, w, g["kkp"], c["ehint"], c["dcv"])
        else:
            Meh = np.zeros((nk, nk), complex)
        VC, E1D = screened_arrays(self.ct, f["Screened"], g["L"], ne, nh)
        z = np.zeros((nk, nk), complex)
        Heh, Hee, Hhh = calc_h(Meh, z, z, C2, D2, p2, VC, c["Ee"], c["Eh"], prm["gap"],
                               f["Excitons"], f["LF"], f["FreePot"])
        GamE = np.full(nk, prm["gam_e"])
        GamH = np.full(nk, prm["gam_h"])
        if f["DiagDph"]:
            GamE = gamma_e(g["kr"], ne, nh, VC, self.dt)
            GamH = gamma_h(g["kr"], ne, nh, VC, self.dt)
        OffP = np.zeros((nk, nk), complex)
        if f["OffDiagDph"]:
            gv = np.array([prm["gam_eh"], prm["gam_e"], prm["gam_h"]])
            OffP, _, _ = offdiag_dephasing2(ne, nh, p2, c["Ee"], c["Eh"], gv, VC)
        # SBEs.py:5203-5226: spontaneous emission rates of the prepared occupations
        Rsp = (spont_emission(ne, nh, c["Ee"], c["Eh"], prm["gap"], VC, self.et)
               if f.get("Recomb", False) else None)
        return dict(Heh=Heh, Hee=Hee, Hhh=Hhh, VC=VC, E1D=E1D, GamE=GamE, GamH=GamH,
                    OffP=OffP, Meh=Meh, Rsp=Rsp)

    def rhs(self, P, C, D, Ex, Ey, Ez, w):
        pr = self.prepare(P, C, D, Ex, Ey, Ez, w)
        z = np.zeros_like(P)
        return (dpdt(C, D, P, pr["Heh"], pr["Hee"], pr["Hhh"], pr["GamE"], pr["GamH"], pr["OffP"]),
                dCdt(C, D, P, pr["Heh"], pr["Hee"], pr["Hhh"], pr["GamE"], pr["GamH"], z),
                dDdt(C, D, P, pr["Heh"], pr["Hee"], pr["Hhh"], pr["GamE"], pr["GamH"], z), pr)

    def rk4_step(self, P, C, D, Ek0, dEk, dt, w):
        """One RK4 step of the batched GPU scheme (no reference counterpart: the
        reference integrates with leapfrog, SBEs.py:5673-5706).

        The occupation-dependent coefficients (screened VC/E1D, GamE/GamH, the
        off-diagonal dephasing matrices De/Dh) are evaluated once from the state at
        the start of the step and held for the four stages; each stage rebuilds
        Meh (field Ek0 + c dEk, c = 0, 1/2, 1/2, 1), the Hartree-Fock Hamiltonians
        and the dephasing contraction from its own state.  After the RK4 update the
        reference's per-step relaxation and charge normalisation are applied
        (SBEs.py:5677-5702) and the sources of the new state are formed.
        Returns (P, C, D, Px, Py, Pz, re, rh); re/rh include x 2 e0 ehint/area.
        """
        f, c, g, prm = self.flags, self.c, self.g, self.p
        nk = g["nk"]
        ne = np.diag(C).copy()
        nh = np.diag(D).copy()
        VC, E1D = screened_arrays(self.ct, f["Screened"], g["L"], ne, nh)
        GamE = np.full(nk, prm["gam_e"])
        GamH = np.full(nk, prm["gam_h"])
        if f["DiagDph"]:
            GamE = gamma_e(g["kr"], ne, nh, VC, self.dt)
            GamH = gamma_h(g["kr"], ne, nh, VC, self.dt)
        Rsp = (spont_emission(ne, nh, c["Ee"], c["Eh"], prm["gap"], VC, self.et)
               if f.get("Recomb", False) else None)
        De = Dh = None
        if f["OffDiagDph"]:
            gv = np.array([prm["gam_eh"], prm["gam_e"], prm["gam_h"]])
            De = offdiag_De(ne, nh, c["Ee"], c["Eh"], gv[0], gv[2], VC)
            Dh = offdiag_Dh(ne, nh, c["Ee"], c["Eh"], gv[1], gv[2], VC)
        z = np.zeros((nk, nk), complex)

        def f_rhs(Ps, Cs, Ds, frac):
            Ek = [Ek0[i] + frac * dEk[i] for i in range(3)]
            Meh = (calc_meh(Ek[0], Ek[1], Ek[2], w, g["kkp"], c["ehint"], c["dcv"])
                   if f["Optics"] else z)
            Heh, Hee, Hhh = calc_h(Meh, z, z, Cs, Ds, Ps, VC, c["Ee"], c["Eh"], prm["gap"],
                                   f["Excitons"], f["LF"], False)
            OffP = offdiag_contract(Dh, De, Ps) if De is not None else z
            return (dpdt(Cs, Ds, Ps, Heh, Hee, Hhh, GamE, GamH, OffP),
                    dCdt(Cs, Ds, Ps, Heh, Hee, Hhh, GamE, GamH, z),
                    dDdt(Cs, Ds, Ps, Heh, Hee, Hhh, GamE, GamH, z))

        X = (P, C, D)
        k1 = f_rhs(*X, 0.0)
        k2 = f_rhs(*[x + 0.5 * dt * k for x, k in zip(X, k1)], 0.5)
        k3 = f_rhs(*[x + 0.5 * dt * k for x, k in zip(X, k2)], 0.5)
        k4 = f_rhs(*[x + dt * k for x, k in zip(X, k3)], 1.0)
        P, C, D = [x + dt / 6.0 * (a + 2.0 * b + 2.0 * cc + d)
                   for x, a, b, cc, d in zip(X, k1, k2, k3, k4)]
        if f["EHs"] or f["Phonon"]:   # SBEs.py:5677 (the Recomb decay is inside)
            ne3, nh3 = relax(np.diag(C).copy(), np.diag(D).copy(), VC, E1D, self.pt, dt,
                             f["EHs"], f["Phonon"], mb=self.mb, rsp=Rsp)
            C[np.diag_indices(nk)] = ne3
            D[np.diag_indices(nk)] = nh3
        if f.get("DCTrans", False):
            # SBEs.py:5686-5690 with the step-start field (q = 0 at index 0)
            eac = np.real(Ek0[0][0])
            dky = g["kr"][2] - g["kr"][1]
            C, D, P = [dc_transport(X, prm.get("Edc", 0.0), eac, dt, dky, f["LF"])
                       for X in (C, D, P)]
        ne3 = np.abs(np.diag(C)).astype(complex)
        nh3 = np.abs(np.diag(D)).astype(complex)
        # carrier numbers before the normalisation (the library's charge record)
        self.last_charge = (float(np.sum(np.abs(ne3))), float(np.sum(np.abs(nh3))))
        total = (np.sum(np.abs(ne3)) + np.sum(np.abs(nh3))) / 2.0
        ne3 = ne3 * total / (np.sum(np.abs(ne3)) + SMALL)
        nh3 = nh3 * total / (np.sum(np.abs(nh3)) + SMALL)
        C[np.diag_indices(nk)] = ne3
        D[np.diag_indices(nk)] = nh3
        Px, Py, Pz, re, rh = self.sources(P, C, D, ne3, nh3, w)
        return P, C, D, Px, Py, Pz, re, rh

    def sources(self, p3, C3, D3, ne3, nh3, w):
        """SBEs.py:5720-5753: QWPolarization3 and QWRho5 (x 2 e0 ehint/area)."""
        g, c, f = self.g, self.c, self.flags
        nr = g["nr"]
        if f["Optics"]:
            Px, Py, Pz = qw_polarization3(g["r"], g["kr"], p3, c["ehint"], c["area"], g["L"], w,
                                          c["dcv"], self.window, self.E)
        else:
            Px = Py = Pz = np.zeros(nr, complex)
        if f["LF"]:
            re, rh = qw_rho5(g["r"], g["L"], C3, D3, ne3, nh3, self.window, self.E)
            re = 2.0 * E0 * re / c["area"] * c["ehint"]
            rh = 2.0 * E0 * rh / c["area"] * c["ehint"]
        else:
            re = rh = np.zeros(nr, complex)
        return Px, Py, Pz, re, rh


class Solver:
    """SBEs.py:4619-5985 SBESolver restated without file output: the state
    YY/CC/DD (Nk, Nk, Nw) x 3 time levels, QWCalculator and the leapfrog step."""

    def __init__(self, nk, L, params, flags, nw, Emax0, temp=77.0):
        self.wire = Wire(nk, L, params, flags, temp)
        self.nw = nw
        self.Emax0 = Emax0
        self.wireoff = True
        nk = self.wire.g["nk"]
        for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
            setattr(self, nm, np.zeros((nk, nk, nw), complex))
        fe = fermi(self.wire.c["Ee"] + params["gap"] / 2.0, temp)
        for w in range(nw):
            for nm in ("CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
                getattr(self, nm)[np.arange(nk), np.arange(nk), w] = fe

    def sbe_calculator(self, Ex, Ey, Ez, dt, w):
        """SBEs.py:5612-5820 _sbe_calculator (numerics only)."""
        wi, f, g = self.wire, self.wire.flags, self.wire.g
        i = w - 1
        p1, p2 = self.YY2[:, :, i].copy(), self.YY3[:, :, i].copy()
        C1, C2 = self.CC2[:, :, i].copy(), self.CC3[:, :, i].copy()
        D1, D2 = self.DD2[:, :, i].copy(), self.DD3[:, :, i].copy()
        dP, dC, dD, pr = wi.rhs(p2, C2, D2, Ex, Ey, Ez, w)
        C3 = C1 + dC * dt * 2.0
        D3 = D1 + dD * dt * 2.0
        p3 = p1 + dP * dt * 2.0
        if f["EHs"] or f["Phonon"]:   # SBEs.py:5677 (the Recomb decay is inside)
            ne3, nh3 = relax(np.diag(C3).copy(), np.diag(D3).copy(), pr["VC"], pr["E1D"],
                             wi.pt, dt, f["EHs"], f["Phonon"], mb=wi.mb, rsp=pr["Rsp"])
            C3[np.diag_indices(g["nk"])] = ne3
            D3[np.diag_indices(g["nk"])] = nh3
        if f.get("DCTrans", False):
            # SBEs.py:5686-5690
            eac = np.real(Ex[g["NQ0"]])
            dky = g["kr"][2] - g["kr"][1]
            C3, D3, p3 = [dc_transport(X, wi.p.get("Edc", 0.0), eac, dt, dky, f["LF"])
                          for X in (C3, D3, p3)]
        ne3 = np.abs(np.diag(C3)).astype(complex)
        nh3 = np.abs(np.diag(D3)).astype(complex)
        total = (np.sum(np.abs(ne3)) + np.sum(np.abs(nh3))) / 2.0
        ne3 = ne3 * total / (np.sum(np.abs(ne3)) + SMALL)
        nh3 = nh3 * total / (np.sum(np.abs(nh3)) + SMALL)
        C3[np.diag_indices(g["nk"])] = ne3
        D3[np.diag_indices(g["nk"])] = nh3
        p2 = (p1 + p3) / 2.0
        C2 = (C1 + C3) / 2.0
        D2 = (D1 + D3) / 2.0
        Px, Py, Pz, re, rh = wi.sources(p3, C3, D3, ne3, nh3, w)
        # SBEs.py:5769-5809: the statistics of info.WW.t.dat and EP.WW.t.dat
        ne2 = np.abs(np.diag(C2)).astype(complex)
        nh2 = np.abs(np.diag(D2)).astype(complex)
        self.last_info = wire_info(ne2, nh2, re, rh, (Ex, Ey, Ez), (Px, Py, Pz), g["kr"],
                                   wi.p["me"], wi.p["mh"], wi.c["Ee"], wi.c["Eh"], wi.p["gap"],
                                   g["L"], PI / g["L"], pr["VC"])   # dkr (SBEs.py:4755)
        self.YY1[:, :, i], self.YY2[:, :, i], self.YY3[:, :, i] = p1, p2, p3
        self.CC1[:, :, i], self.CC2[:, :, i], self.CC3[:, :, i] = C1, C2, C3
        self.DD1[:, :, i], self.DD2[:, :, i], self.DD3[:, :, i] = D1, D2, D3
        return Px, Py, Pz, re, rh

    def qw_calculator(self, Exx, Eyy, Ezz, Vrr, rr, dt, w):
        """SBEs.py:5826-5985 QWCalculator: returns (Pxx, Pyy, Pzz, Rho)."""
        n = len(rr)
        zero = np.zeros(n, complex)
        mag = np.max(np.sqrt(np.abs(Exx) ** 2 + np.abs(Eyy) ** 2 + np.abs(Ezz) ** 2))
        if self.wireoff and mag < 1e-3 * self.Emax0:
            return zero, zero.copy(), zero.copy(), zero.copy()
        self.wireoff = False
        wi = self.wire
        Ex, Ey, Ez, Vr = prop2qw(rr, Exx, Eyy, Ezz, Vrr, wi.g["r"], wi.window)
        Px, Py, Pz, re, rh = self.sbe_calculator(Ex, Ey, Ez, dt, w)
        Pxx, Pyy, Pzz, RhoE, RhoH = qw2prop(wi.g["r"], Px, Py, Pz, re, rh, rr, wi.flags["LF"])
        return Pxx, Pyy, Pzz, RhoH - RhoE
