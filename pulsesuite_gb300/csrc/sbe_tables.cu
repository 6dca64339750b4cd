// One-time FP64 tables of every wire, built on the device.
//
// This translation unit is compiled with -fmad=false so that products and sums
// round exactly as the reference's NumPy expressions do (index maps that round
// a quotient to the nearest integer depend on it).
#include "sbe_ctx.cuh"

#include <cmath>

namespace sbe {

// coulomb.py:39-66 _K03_jit, kept as written (a truncated series and only the
// leading asymptotic term; this is what the reference's V(q) tables use).
__device__ double k0_truncated(double x) {
  if (x > 100.0) return 0.0;
  if (x < 1e-10) return 23.0;
  if (x < 2.0) {
    double x2 = x * x;
    double res = -log(0.5 * x) - kEuler;
    double term = 1.0;
    for (int k = 1; k < 20; ++k) {
      term = term * 0.25 * x2 / (double)(k * k);
      res = res + term * (1.0 / k - kEuler);
      if (fabs(term) < 1e-15) break;
    }
    return res;
  }
  return sqrt(kPi / (2.0 * x)) * exp(-x);
}

__device__ double dfact2(int n) {
  double r = 1.0;
  while (n > 1) { r *= n; n -= 2; }
  return r;
}

// Zhang & Jin CIK01 asymptotic coefficients from their closed forms:
// I0 ~ e^z/sqrt(2 pi z) sum a_k z^-k, a_k = ((2k-1)!!)^2 / (k! 8^k);
// I0 K0 ~ 1/(2z) sum b_k z^-2k,       b_k = ((2k-1)!!)^3 / ((2k)!! 4^k).
__device__ double i0_asy_coef(int k) {
  double f = 1.0;
  for (int j = 2; j <= k; ++j) f *= j;
  double d = dfact2(2 * k - 1);
  return d * d / (f * pow(8.0, (double)k));
}
__device__ double k0i0_asy_coef(int k) {
  double d = dfact2(2 * k - 1);
  return d * d * d / (dfact2(2 * k) * pow(4.0, (double)k));
}

// usefulsubs.py:1700-1730: I0 for real x (series for x <= 18, else asymptotic).
// The reference runs this in NumPy complex128, whose division multiplies by the
// divisor's reciprocal; the same is done here.
__device__ double i0_cik(double x) {
  if (x <= 18.0) {
    double s = 1.0, cr = 1.0, x2 = x * x;
    for (int k = 1; k <= 50; ++k) {
      cr = 0.25 * cr * x2 * (1.0 / (double)(k * k));
      s = s + cr;
      if (fabs(cr * (1.0 / s)) < 1e-15) break;
    }
    return s;
  }
  int k0 = x < 35.0 ? 12 : (x < 50.0 ? 9 : 7);
  double ca = exp(x) / sqrt(2.0 * kPi * x);
  double s = 1.0, zr = 1.0 / x;
  for (int k = 1; k <= k0; ++k) s = s + i0_asy_coef(k) * pow(zr, (double)k);
  return ca * s;
}

// usefulsubs.py:1649-1800 K03 (real K0 of cik01).
__device__ double k0_cik(double x) {
  if (x > 1e2) return 0.0;
  if (x == 0.0) return 1e30;
  if (x <= 9.0) {
    double cs = 0.0, ct = -log(0.5 * x) - kEuler, w0 = 0.0, cr = 1.0, cw = 0.0, x2 = x * x;
    for (int k = 1; k <= 50; ++k) {
      w0 = w0 + 1.0 / k;
      cr = 0.25 * cr * (1.0 / (double)(k * k)) * x2;
      cs = cs + cr * (w0 + ct);
      if (fabs((cs - cw) * (1.0 / cs)) < 1e-15) break;
      cw = cs;
    }
    return ct + cs;
  }
  double cb = 0.5 * (1.0 / x), zr2 = 1.0 / (x * x), s = 1.0;
  for (int k = 1; k <= 10; ++k) s = s + k0i0_asy_coef(k) * pow(zr2, (double)k);
  return cb * s * (1.0 / i0_cik(x));
}

// ---------------------------------------------------------------------------
// Grid: kr (SBEs.py:5028-5040), r = linspace(-L, L, Nr) (typespace.py:815),
// Ee, Eh (SBEs.py:4822-4823), Vxx2 index iq (dephasing.py:362-378), xe/xh
// (dephasing.py:499-500).
__global__ void k_grid(const WireDev* wires, double* kr, double* r, double* Ee, double* Eh,
                       int* iq, double* xeh) {
  const WireDev W = wires[blockIdx.y];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < W.nk) {
    double v = W.dkr * ((double)(i - W.dnk) - 0.5);
    kr[W.off_vec + i] = v;
    double h2 = kHbar * kHbar;
    Ee[W.off_vec + i] = h2 * (v * v) / (2.0 * W.me);
    Eh[W.off_vec + i] = h2 * (v * v) / (2.0 * W.mh);
    double k0 = W.dkr * ((double)(0 - W.dnk) - 0.5);
    double k1 = W.dkr * ((double)(1 - W.dnk) - 0.5);
    double dq = W.nk > 1 ? k1 - k0 : 1.0;
    iq[W.off_vec + i] = (int)rint(fabs(v / dq));
    double av = fabs(v);
    double den = av + dq * 1e-5;
    xeh[2 * W.off_vec + i] = W.me / h2 * av / (den * den) / dq;
    xeh[2 * W.off_vec + W.nk + i] = W.mh / h2 * av / (den * den) / dq;
  }
  if (i < W.nr) {
    double start = -(2.0 * W.L) / 2.0, stop = (2.0 * W.L) / 2.0;
    double step = (stop - start) / (double)(W.nr - 1);
    double v = (double)i * step + start;
    if (i == W.nr - 1) v = stop;
    r[W.off_r + i] = v;
  }
}

// Vint (coulomb.py:70-104) regrouped: the double sum over (i, j) of
// exp(-(a1 y_i)^2) exp(-(a2 y_j)^2) K0t(dk sqrt((y_i-y_j)^2 + D0^2)) depends on
// i-j through K0t only, so corr[m] = sum_{i-j=m} ea_i eb_j is formed once and
// each V(Q) is a sum over m.
__global__ void k_vcorr(const WireDev* wires, const double* r, double* vcorr) {
  const WireDev W = wires[blockIdx.y];
  int n = blockIdx.z;  // 0 eh, 1 ee, 2 hh
  double a1 = (n == 2) ? W.alphah : W.alphae;
  double a2 = (n == 1) ? W.alphae : W.alphah;
  int N1 = W.nr / 4, N2 = 3 * W.nr / 4, N = N2 - N1 + 1;
  double* out = vcorr + 3 * (W.off_r + 2 * blockIdx.y) + (long long)n * (W.nr + 2);
  const double* y = r + W.off_r + N1;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < 2 * N - 1; m += gridDim.x * blockDim.x) {
    int dm = m - (N - 1);  // i - j
    double s = 0.0;
    int i0 = dm > 0 ? dm : 0;
    int i1 = dm > 0 ? N - 1 : N - 1 + dm;
    for (int i = i0; i <= i1; ++i) {
      int j = i - dm;
      double ai = a1 * y[i], bj = a2 * y[j];
      s += exp(-(ai * ai) - (bj * bj));
    }
    out[m] = s;
  }
}

__global__ void k_vtab(const WireDev* wires, const double* r, const double* vcorr, double* v0) {
  const WireDev W = wires[blockIdx.z];
  int d = blockIdx.x;
  int n = blockIdx.y;
  if (d >= W.nk) return;
  double a1 = (n == 2) ? W.alphah : W.alphae;
  double a2 = (n == 1) ? W.alphae : W.alphah;
  int N1 = W.nr / 4, N2 = 3 * W.nr / 4, N = N2 - N1 + 1;
  const double* cor = vcorr + 3 * (W.off_r + 2 * blockIdx.z) + (long long)n * (W.nr + 2);
  const double* y = r + W.off_r;
  double dyy = y[1] - y[0];
  // Qr (GetKArray rolled): ((d + Nr/2) dk) - ((Nr/2) dk) with dk = 2 pi / (2 L)
  double dk = kTwoPi / (2.0 * W.L);
  double Q = (double)(d + W.nr / 2) * dk - (double)(W.nr / 2) * dk;
  double kmin = (a1 + a2) / 4.0;
  double dq = fmax(fabs(Q), kmin);
  double mult = a1 * a2 / kPi * (dyy * dyy);
  double s = 0.0;
  for (int m = threadIdx.x; m < 2 * N - 1; m += blockDim.x) {
    int dm = m - (N - 1);
    double dyv = y[N1 + (dm > 0 ? dm : 0)] - y[N1 + (dm > 0 ? 0 : -dm)];
    double rr = sqrt(dyv * dyv + W.Delta0 * W.Delta0);
    s += cor[m] * k0_truncated(dq * rr);
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double pref = kE0 * kE0 / (kTwoPi * kEps0 * W.epsr * W.L);
    v0[3 * W.off_vec + (long long)n * W.nk + d] = pref * (mult * red[0]);
  }
}

// coulomb.py:302-330 MakeQs and 580-630 CalcChi1D, by |k1-k2|.
__global__ void k_chi(const WireDev* wires, const double* kr, double* qeh, double* chi) {
  const WireDev W = wires[blockIdx.y];
  int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= W.nk) return;
  const double* k = kr + W.off_vec;
  double dif = fabs(k[d] - k[0]);
  double qe = fmax(dif, W.alphae / 2.0);
  double qh = fmax(dif, W.alphah / 2.0);
  double Re = sqrt((2.0 / W.alphae) * (2.0 / W.alphae) + W.Delta0 * W.Delta0);
  double Rh = sqrt((2.0 / W.alphah) * (2.0 / W.alphah) + W.Delta0 * W.Delta0);
  double scale = kE0 * kE0 / (kTwoPi * kEps0 * W.epsr * (kHbar * kHbar));
  qeh[2 * W.off_vec + d] = qe;
  qeh[2 * W.off_vec + W.nk + d] = qh;
  chi[2 * W.off_vec + d] = W.me * k0_cik(qe * Re) / qe * scale;
  chi[2 * W.off_vec + W.nk + d] = W.mh * k0_cik(qh * Rh) / qh * scale;
}

// phonons.py:55-136 InitializePhonons: EP, HP (the 2 Gph factor and the k != k1 mask).
__global__ void k_phonon(const WireDev* wires, const double* Ee, const double* Eh, double* EP,
                         double* HP) {
  const WireDev W = wires[blockIdx.z];
  int k1 = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (k >= W.nk || k1 >= W.nk) return;
  const double* e = Ee + W.off_vec;
  const double* h = Eh + W.off_vec;
  double hO = kHbar * W.Oph, hG = kHbar * W.Gph, N0 = W.n0ph;
  double de = e[k] - e[k1], dh = h[k] - h[k1];
  double ep = N0 / ((de - hO) * (de - hO) + hG * hG) + (N0 + 1.0) / ((de + hO) * (de + hO) + hG * hG);
  double hp = N0 / ((dh - hO) * (dh - hO) + hG * hG) + (N0 + 1.0) / ((dh + hO) * (dh + hO) + hG * hG);
  double idel = (k == k1) ? 0.0 : 1.0;
  EP[W.off_mat + (long long)k * W.nk + k1] = ep * 2.0 * W.Gph * idel;
  HP[W.off_mat + (long long)k * W.nk + k1] = hp * 2.0 * W.Gph * idel;
}

// dephasing.py:472-535 InitializeDephasing index maps [k][q].
__global__ void k_deph_maps(const WireDev* wires, const double* kr, int* maps) {
  const WireDev W = wires[blockIdx.z];
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (k >= W.nk || q >= W.nk) return;
  const double* ky = kr + W.off_vec;
  int nk = W.nk;
  double dk = nk > 1 ? ky[1] - ky[0] : 1.0;
  double kmax = ky[nk - 1] + dk, kmin = ky[0] - dk;
  int nk0 = (nk - 1) / 2 + 1;
  auto idx = [&](double v) {
    double c = fmin(fmax(v, kmin), kmax);
    return (int)rint(c / dk) + nk0 - 1;
  };
  long long base = 6 * W.off_mat + (long long)k * nk + q;
  long long st = (long long)nk * nk;
  double kk = ky[k], qq = ky[q];
  maps[base + 0 * st] = idx(kk + qq);
  maps[base + 1 * st] = idx(kk - qq);
  double k1p0 = ((W.me + W.mh) * qq - 2.0 * W.mh * kk) / 2.0 / W.me;
  maps[base + 2 * st] = idx(k1p0);
  maps[base + 3 * st] = idx(k1p0 - qq);
  double k10 = ((W.me + W.mh) * qq - 2.0 * W.me * kk) / 2.0 / W.mh;
  maps[base + 4 * st] = idx(k10);
  maps[base + 5 * st] = idx(k10 - qq);
}

// qwoptics.py:628-663 CalcQWWindow, CalcExpikr; FFTG of the window (the wire-k
// field of a spatially uniform unit field, usefulsubs.py:2245).
__global__ void k_optics(const WireDev* wires, const double* kr, const double* r, double* win,
                         double2* expikr) {
  const WireDev W = wires[blockIdx.z];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (j >= W.nr) return;
  double rj = r[W.off_r + j];
  if (k == 0) win[W.off_r + j] = exp(-pow(rj / (W.L / 2.0), 150.0));
  if (k < W.nk) {
    double ph = kr[W.off_vec + k] * rj;
    double s, c;
    sincos(ph, &s, &c);
    expikr[W.off_kr + (long long)k * W.nr + j] = make_double2(c, s);
  }
}

__global__ void k_window_fft(const WireDev* wires, const double* win, double2* wk) {
  const WireDev W = wires[blockIdx.y];
  int q = blockIdx.x;
  if (q >= W.nr) return;
  double sr = 0.0, si = 0.0;
  for (int j = threadIdx.x; j < W.nr; j += blockDim.x) {
    long long qj = ((long long)q * j) % W.nr;
    double s, c;
    sincospi(-2.0 * (double)qj / (double)W.nr, &s, &c);
    double v = win[W.off_r + j];
    sr += v * c;
    si += v * s;
  }
  __shared__ double rr[128], ri[128];
  rr[threadIdx.x] = sr;
  ri[threadIdx.x] = si;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      rr[threadIdx.x] += rr[threadIdx.x + o];
      ri[threadIdx.x] += ri[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) wk[W.off_r + q] = make_double2(-rr[0] / W.nr, -ri[0] / W.nr);
}

int build_tables(SbeCtx* c, cudaStream_t s) {
  int nw = c->nw;
  dim3 b(256);
  int gk = (std::max(c->nk_max, c->nr_max) + 255) / 256;
  k_grid<<<dim3(gk, nw), b, 0, s>>>(c->d_wires, c->kr, c->r, c->Ee, c->Eh, c->iq, c->xeh);
  k_vcorr<<<dim3(8, nw, 3), b, 0, s>>>(c->d_wires, c->r, c->vcorr);
  k_vtab<<<dim3(c->nk_max, 3, nw), b, 0, s>>>(c->d_wires, c->r, c->vcorr, c->v0);
  k_chi<<<dim3((c->nk_max + 127) / 128, nw), 128, 0, s>>>(c->d_wires, c->kr, c->qeh, c->chi);
  k_phonon<<<dim3((c->nk_max + 127) / 128, c->nk_max, nw), 128, 0, s>>>(c->d_wires, c->Ee, c->Eh,
                                                                        c->EP, c->HP);
  k_deph_maps<<<dim3((c->nk_max + 127) / 128, c->nk_max, nw), 128, 0, s>>>(c->d_wires, c->kr,
                                                                          c->maps);
  k_optics<<<dim3((c->nr_max + 127) / 128, std::max(c->nk_max, 1), nw), 128, 0, s>>>(
      c->d_wires, c->kr, c->r, c->window, c->expikr);
  k_window_fft<<<dim3(c->nr_max, nw), 128, 0, s>>>(c->d_wires, c->window, c->wk);
  return cuda_check(cudaGetLastError(), "table kernels");
}

}  // namespace sbe
