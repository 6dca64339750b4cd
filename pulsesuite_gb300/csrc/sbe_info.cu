// Per-step statistics of one wire (SBEs.py:5769-5809): the columns after the time of
// dataQW/info.WW.t.dat and dataQW/EP.WW.t.dat, reduced on the device from the
// occupations of the middle level (ne2 = |C2_kk|, nh2 = |D2_kk|), the step's
// screened interaction, the real-space sources and the wire-k field.  The host
// formats the line.  Helpers restated: CalcVD (dcfield.py:128-151), CalcI0
// (:1110-1148) with EkReNorm (:339-344) and DriftVt (:348-359), CalcI0n (:103-125),
// TotalEnergy / Temperature (usefulsubs.py:1185-1253); GetEDrift is the DC module's
// ERate, which SBEs never sets (0).
#include <cmath>

#include "sbe_ctx.cuh"
#include "sbe_internal.cuh"

namespace sbe {
namespace {

constexpr int kInfoThreads = 256;

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kInfoThreads / 32; ++i) s += red[i];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

__device__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int i = 1; i < kInfoThreads / 32; ++i) m = fmax(m, red[i]);
    red[32] = m;
  }
  __syncthreads();
  return red[32];
}

// Ec(k) = E(k) + sum_k' n(k') (V[k][k] - V[k][k']) / 2 with the screened matrix of
// the preparation, V[k][k'] = v(k - k') for k >= k', else 0
__device__ void ek_renorm(int nk, const double* n, const double* E, const double* v, double sn,
                          double* Ec) {
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    double s = 0.0;
    for (int kp = 0; kp <= k; ++kp) s += n[kp] * v[k - kp];
    Ec[k] = E[k] + (v[0] * sn - s) / 2.0;
  }
  __syncthreads();
}

// DriftVt: <dEc/dk> / hbar with centred differences and linear ends
__device__ double drift_vt(int nk, const double* n, const double* Ec, double dkk, double sn,
                           double* red) {
  auto dedk = [&](int i) { return (Ec[i + 1] - Ec[i - 1]) / 2.0 / dkk; };
  double s = 0.0;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    double d;
    if (k == 0) d = 2.0 * dedk(1) - dedk(2);
    else if (k == nk - 1) d = 2.0 * dedk(nk - 2) - dedk(nk - 3);
    else d = dedk(k);
    s += d * n[k];
  }
  return block_sum(s, red) / (1e-100 + sn) / kHbar;
}

__global__ void __launch_bounds__(kInfoThreads) k_wire_info(const WireDev* wires, int w,
                                                            const double2* C2, const double2* D2,
                                                            const double* vs, const double* Ee,
                                                            const double* Eh, const double* kr,
                                                            const double2* src, const double2* Ek,
                                                            double* out) {
  extern __shared__ double sh[];
  __shared__ double red[33];
  const WireDev W = wires[w];
  const int nk = W.nk, nr = W.nr;
  double* a = sh;            // ne2
  double* b = sh + nk;       // nh2
  double* ec = sh + 2 * nk;  // renormalised energies
  const double* ke = kr + W.off_vec;
  const double* ee = Ee + W.off_vec;
  const double* eh = Eh + W.off_vec;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    const long long o = W.off_mat + (long long)k * nk + k;
    a[k] = hypot(C2[o].x, C2[o].y);
    b[k] = hypot(D2[o].x, D2[o].y);
  }
  __syncthreads();
  double t[12] = {};
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    const double q = ke[k];
    t[0] += a[k] * kHbar * q / W.me;
    t[1] += a[k] + 1e-200;
    t[2] += b[k] * kHbar * q / W.mh;
    t[3] += b[k] + 1e-200;
    t[4] += a[k];
    t[5] += b[k];
    t[6] += a[k] * (ee[k] + W.gap);
    t[7] += b[k] * eh[k];
    t[8] += a[k] * ee[k];
    t[9] += (a[k] - b[k]) * q;
    t[10] += a[k] * q;
    t[11] += b[k] * q;
  }
  double s[12];
  for (int i = 0; i < 12; ++i) s[i] = block_sum(t[i], red);
  double i1 = 0.0, i2 = 0.0;   // CalcI0n sums: ne kr, (1 - nh) kr
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    i1 += a[k] * ke[k] * kHbar / W.me;
    i2 += (1.0 - b[k]) * ke[k] * kHbar / (-W.mh);
  }
  i1 = block_sum(i1, red);
  i2 = block_sum(i2, red);
  double tb = 0.0;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) tb += b[k] * eh[k];
  tb = block_sum(tb, red);
  // max |Re|, |Rh| over the wire-k arrays the reference holds (FFTG = -fft / Nr of
  // the real-space sources kept here): one direct DFT row per q, exact twiddles
  double mre = 0.0, mrh = 0.0;
  const double2* re = src + 5LL * W.off_r + 3LL * nr;
  const double2* rh = re + nr;
  for (int q = threadIdx.x; q < nr; q += blockDim.x) {
    double2 fe = make_double2(0.0, 0.0), fh = make_double2(0.0, 0.0);
    for (int j = 0; j < nr; ++j) {
      const long long m = ((long long)q * j) % nr;
      double sn, cs;
      sincospi(-2.0 * (double)m / (double)nr, &sn, &cs);
      fe.x += re[j].x * cs - re[j].y * sn;
      fe.y += re[j].x * sn + re[j].y * cs;
      fh.x += rh[j].x * cs - rh[j].y * sn;
      fh.y += rh[j].x * sn + rh[j].y * cs;
    }
    mre = fmax(mre, hypot(fe.x, fe.y) / nr);
    mrh = fmax(mrh, hypot(fh.x, fh.y) / nr);
  }
  mre = block_max(mre, red);
  mrh = block_max(mrh, red);
  // iFFTG(E)[Nr/2] = -sum_q (-1)^q E_q (Nr even)
  double ex[3];
  for (int c = 0; c < 3; ++c) {
    const double2* e = Ek + 3LL * W.off_r + (long long)c * nr;
    double acc = 0.0;
    for (int q = threadIdx.x; q < nr; q += blockDim.x) acc += (q & 1) ? e[q].x : -e[q].x;
    ex[c] = block_sum(acc, red);
  }
  // CalcI0: drift velocities of the renormalised bands
  const double* veh = vs + 3 * W.off_vec;
  const double dkr = kPi / W.L;
  ek_renorm(nk, a, ee, veh + nk, s[4], ec);
  const double ve = drift_vt(nk, a, ec, dkr, s[4], red);
  ek_renorm(nk, b, eh, veh + 2 * nk, s[5], ec);
  const double vh = drift_vt(nk, b, ec, dkr, s[5], red);
  if (threadIdx.x == 0) {
    const double dk = nk > 1 ? ke[1] - ke[0] : 1.0;
    out[0] = s[0] / s[1];
    out[1] = s[2] / s[3];
    out[2] = 2.0 * s[4] / W.L;
    out[3] = 2.0 * s[5] / W.L;
    out[4] = s[6] / kE0;
    out[5] = s[7] / kE0;
    out[6] = 2.0 * (s[8] / (s[4] + 1e-100)) / kKb;
    out[7] = 2.0 * (tb / (s[5] + 1e-100)) / kKb;
    out[8] = mre;
    out[9] = mrh;
    out[10] = 0.0;
    out[11] = kHbar * s[9] * 2.0;
    out[12] = kHbar * s[10];
    out[13] = -kHbar * s[11];
    out[14] = -kE0 * (ve + vh) * s[4] * dkr * 2.0;
    out[15] = -kE0 * i1 * 2.0 * dk;
    out[16] = -kE0 * i2 * 2.0 * dk;
    for (int c = 0; c < 3; ++c) {
      out[17 + c] = ex[c];
      out[20 + c] = src[5LL * W.off_r + (long long)c * nr + nr / 2].x;
    }
  }
}

// Re iFFTG(E_c)(r) of the wire-k field (usefulsubs.py:2271-2294: iFFTG(F) = -N
// ifft(F) = -sum_q F[q] e^{+2 pi i q r / N}): one block per (r, component)
__global__ void k_wire_field_r(const WireDev* wires, int w, const double2* Ek, double* er) {
  const WireDev W = wires[w];
  const int nr = W.nr, r = blockIdx.x, c = blockIdx.y;
  const double2* e = Ek + 3LL * W.off_r + (long long)c * nr;
  double acc = 0.0;
  for (int q = threadIdx.x; q < nr; q += blockDim.x) {
    const long long qr = ((long long)q * r) % nr;
    double sn, cs;
    sincospi(2.0 * (double)qr / (double)nr, &sn, &cs);
    acc += e[q].x * cs - e[q].y * sn;
  }
  __shared__ double red[33];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) er[(long long)c * nr + r] = -t;
}

// sum_c sum_r (Re P_c(r) - P0_c(r)) Re E_c(r): the wire-grid increment of the
// reference's EPEnergyW (SBEs.py:5950-5958) before its 0.5 dr area factor
__global__ void k_wire_pdote(const WireDev* wires, int w, const double2* src, const double* P0,
                             const double* er, double* out) {
  const WireDev W = wires[w];
  const int nr = W.nr;
  double acc = 0.0;
  for (int c = 0; c < 3; ++c) {
    const double2* pc = src + 5LL * W.off_r + (long long)c * nr;
    for (int r = threadIdx.x; r < nr; r += blockDim.x) {
      const double p0 = P0 ? P0[(long long)c * nr + r] : 0.0;
      acc += (pc[r].x - p0) * er[(long long)c * nr + r];
    }
  }
  __shared__ double red[33];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) *out = t;
}

// max and min of Re De and Re Dh of wire w (dephasing.py:731-740), [2Nk+1][Nk] each
__global__ void k_deph_extrema(const WireDev* wires, int w, const double* De, const double* Dh,
                               double* out4) {
  const WireDev W = wires[w];
  const long long n = (long long)(2 * W.nk + 1) * W.nk;
  const double* a[2] = {De + W.off_dd, Dh + W.off_dd};
  __shared__ double red[33];
  for (int i = 0; i < 2; ++i) {
    double mx = -INFINITY, mn = INFINITY;
    for (long long j = threadIdx.x; j < n; j += blockDim.x) {
      mx = fmax(mx, a[i][j]);
      mn = fmin(mn, a[i][j]);
    }
    mx = block_max(mx, red);
    mn = -block_max(-mn, red);
    if (threadIdx.x == 0) {
      out4[2 * i] = mx;
      out4[2 * i + 1] = mn;
    }
  }
}

}  // namespace

int launch_wire_pdote(SbeCtx* c, int w, const double2* Ek, const double2* src, const double* P0,
                      double* out, cudaStream_t s) {
  const int nr = c->wires[w].nr;
  double* er = reinterpret_cast<double*>(c->qscr);   // 3 nr doubles of the scratch
  k_wire_field_r<<<dim3(nr, 3), kInfoThreads, 0, s>>>(c->d_wires, w, Ek, er);
  k_wire_pdote<<<1, kInfoThreads, 0, s>>>(c->d_wires, w, src, P0, er, out);
  return cuda_check(cudaGetLastError(), "sbe_wire_pdote");
}

int launch_deph_extrema(SbeCtx* c, int w, double* out4, cudaStream_t s) {
  k_deph_extrema<<<1, kInfoThreads, 0, s>>>(c->d_wires, w, c->De, c->Dh, out4);
  return cuda_check(cudaGetLastError(), "sbe_deph_extrema");
}

int launch_wire_info(SbeCtx* c, int w, const double2* C2, const double2* D2, const double2* src,
                     const double2* Ek, double* out, cudaStream_t s) {
  const int nk = c->wires[w].nk;
  const size_t smem = sizeof(double) * 3 * (size_t)nk;
  if (smem > 200 * 1024) return fail(SBE_ERR_UNSUPPORTED, "sbe_wire_info: Nk too large");
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_wire_info, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_wire_info<<<1, kInfoThreads, smem, s>>>(c->d_wires, w, C2, D2, c->vs, c->Ee, c->Eh, c->kr,
                                            src, Ek, out);
  return cuda_check(cudaGetLastError(), "sbe_wire_info");
}

}  // namespace sbe
