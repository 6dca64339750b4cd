// Carrier-carrier scattering rates (flag EHs): MBCE / MBCH of coulomb.py:957-1071
// (called by RelaxationE / RelaxationH, SBEs.py:1709-1835) with the values of the
// CalcMBArrays tables (coulomb.py:367-499) evaluated where they are used instead
// of stored as three (Nk+1)^3 arrays.
#include "sbe_ctx.cuh"
#include "sbe_internal.cuh"
#include "fp_bits.cuh"

namespace sbe {

namespace {

// CalcMBArrays for 0-based (a, b, d) of the builder (kind 0: Ceh, 1: Cee, 2: Chh):
// k30 = d + b - a (eh) or a + b - d (ee, hh); UnDel[a+1][d+1] UnDel[b+1][k30+1]
// is (a != d); zero where k30 leaves [0, Nk).  Lorentzian 2 g / (E^2 + (hbar g)^2)
// or (2 pi / hbar) GaussDelta(E, hbar g) (coulomb.py:245-262), g = (ge + gh) / 2 for
// eh.  Operations in the reference's order.
__device__ __forceinline__ double mb_value64(int kind, int a, int b, int d, int n,
                                             const double* Ee, const double* Eh, double ge,
                                             double gh, bool lorentz) {
  if (a < 0 || b < 0 || d < 0 || a == d) return 0.0;
  const int c = kind == 0 ? d + b - a : a + b - d;
  if (c < 0 || c >= n) return 0.0;
  double E, g;
  if (kind == 0) {
    E = ((Ee[a] + Eh[b]) - Eh[c]) - Ee[d];
    g = (ge + gh) / 2.0;
  } else if (kind == 1) {
    E = ((Ee[a] + Ee[b]) - Ee[c]) - Ee[d];
    g = ge;
  } else {
    E = ((Eh[a] + Eh[b]) - Eh[c]) - Eh[d];
    g = gh;
  }
  const double hg = kHbar * g;
  if (lorentz) return 2.0 * g / (E * E + hg * hg);
  const double x = E / hg;
  return kTwoPi / kHbar * (1.0 / (sqrt(kPi) * hg) * exp(-(x * x)));
}

// Table entry C[x][y][z] as the scattering loops read it: the loops index the
// 1-based table with k - 1, so storage index x holds the builder's x - 1 (a quirk
// of the reference, kept) and index 0 is zero.
__device__ __forceinline__ double mb_store64(int kind, int x, int y, int z, int n,
                                             const double* Ee, const double* Eh, double ge,
                                             double gh, bool lorentz) {
  return mb_value64(kind, x - 1, y - 1, z - 1, n, Ee, Eh, ge, gh, lorentz);
}

// VC[i][j]^2 of the screened tables: the reference's V(q) arrays are lower
// triangular on its grid (V[k1][k2] = v[k1 - k2] for k1 >= k2, else 0), and the
// context keeps v by k1 - k2 >= 0.
__device__ __forceinline__ double vsq_at(const double* v2, int i, int j) {
  return i >= j ? v2[i - j] : 0.0;
}

// One block per (row, wire, species): species 0 electrons (MBCE, row k), 1 holes
// (MBCH, row kp); the threads walk the Nk^2 pairs (q1, q2) of the row; the block
// sums (fixed tree) are added to wrate (Win, Wout of the species).
__global__ void __launch_bounds__(256) k_mbc_rates64(const WireDev* wires, int w_only,
                                                     const double2* nev, const double2* nhv,
                                                     const double* vs, const double* Ee,
                                                     const double* Eh, double* wrate,
                                                     int all) {
  const WireDev W = wires[w_only >= 0 ? w_only : blockIdx.y];
  const int n = W.nk;
  const int row = blockIdx.x + 1;   // 1-based k (electrons) or kp (holes)
  if (row > n || !(all || (W.flags & SBE_F_EHS))) return;
  const bool holes = blockIdx.z == 1;
  extern __shared__ double sh[];
  double* ne = sh;              // [0, n]: 1-based occupations, ne[0] = 0
  double* nh = sh + (n + 1);
  double* v2 = sh + 2 * (n + 1);   // [3][n]: VC^2 by k1 - k2 >= 0 (eh, ee, hh)
  for (int i = threadIdx.x; i <= n; i += blockDim.x) {
    ne[i] = i == 0 ? 0.0 : fabs(nev[W.off_vec + i - 1].x);
    nh[i] = i == 0 ? 0.0 : fabs(nhv[W.off_vec + i - 1].x);
  }
  for (int i = threadIdx.x; i < 3 * n; i += blockDim.x) {
    const double v = vs[3 * W.off_vec + i];
    v2[i] = v * v;
  }
  __syncthreads();
  const double* E_e = Ee + W.off_vec;
  const double* E_h = Eh + W.off_vec;
  const double ge = W.gam_e, gh = W.gam_h;
  const bool lz = (W.flags & SBE_F_LORENTZ) != 0;
  const double* veh = v2;
  const double* vxx = v2 + (holes ? 2 : 1) * n;
  double win = 0.0, wout = 0.0;
  const long long npair = (long long)n * n;
  for (long long p = threadIdx.x; p < npair; p += blockDim.x) {
    const int q1 = (int)(p / n) + 1, q2 = (int)(p % n) + 1;
    if (!holes) {
      const int k = row;
      {
        const int kp = q1, k1 = q2;
        const int k1p = kp + k1 - k;
        if (k1p >= 1 && k1p <= n) {
          const double cv = mb_store64(0, k - 1, kp - 1, k1 - 1, n, E_e, E_h, ge, gh, lz);
          win += vsq_at(veh, k, k1) * (1.0 - nh[kp]) * nh[k1p] * ne[k1] * cv;
        }
        const int k1q = kp + k - k1;
        if (k1q >= 1 && k1q <= n) {
          const double cv = mb_store64(0, k1 - 1, kp - 1, k - 1, n, E_e, E_h, ge, gh, lz);
          wout += vsq_at(veh, k1, k) * (1.0 - ne[k1]) * (1.0 - nh[kp]) * nh[k1q] * cv;
        }
      }
      {
        const int k2 = q1, k4 = q2;
        const int k30 = k + k2 - k4;
        if (k30 >= 1 && k30 <= n) {
          const double cv = mb_store64(1, k - 1, k2 - 1, k4 - 1, n, E_e, E_h, ge, gh, lz);
          win += vsq_at(vxx, k, k4) * (1.0 - ne[k2]) * ne[k30] * ne[k4] * cv;
        }
        const int k31 = k4 + k2 - k;
        if (k31 >= 1 && k31 <= n) {
          const double cv = mb_store64(1, k4 - 1, k2 - 1, k - 1, n, E_e, E_h, ge, gh, lz);
          wout += vsq_at(vxx, k4, k) * (1.0 - ne[k4]) * (1.0 - ne[k2]) * ne[k31] * cv;
        }
      }
    } else {
      const int kp = row;
      {
        const int k = q1, k1 = q2;
        const int k1p = kp + k1 - k;
        if (k1p >= 1 && k1p <= n) {
          const double cv = mb_store64(0, k - 1, kp - 1, k1 - 1, n, E_e, E_h, ge, gh, lz);
          win += vsq_at(veh, k, k1) * (1.0 - ne[k]) * nh[k1p] * ne[k1] * cv;
        }
        const int k1q = kp + k - k1;
        if (k1q >= 1 && k1q <= n) {
          const double cv = mb_store64(0, k - 1, k1q - 1, k1 - 1, n, E_e, E_h, ge, gh, lz);
          wout += vsq_at(veh, k1, k) * (1.0 - ne[k]) * (1.0 - nh[k1q]) * ne[k1] * cv;
        }
      }
      {
        const int k2p = q1, k4p = q2;
        const int k3p = kp + k2p - k4p;
        if (k3p >= 1 && k3p <= n) {
          const double cv = mb_store64(2, kp - 1, k2p - 1, k4p - 1, n, E_e, E_h, ge, gh, lz);
          win += vsq_at(vxx, kp, k4p) * (1.0 - nh[k2p]) * nh[k3p] * nh[k4p] * cv;
        }
        const int k3q = k4p + k2p - kp;
        if (k3q >= 1 && k3q <= n) {
          const double cv = mb_store64(2, k4p - 1, k2p - 1, kp - 1, n, E_e, E_h, ge, gh, lz);
          wout += vsq_at(vxx, k4p, kp) * (1.0 - nh[k4p]) * (1.0 - nh[k2p]) * nh[k3q] * cv;
        }
      }
    }
  }
  __shared__ double red[2][256];
  red[0][threadIdx.x] = win;
  red[1][threadIdx.x] = wout;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* wr = wrate + 4 * W.off_vec + (holes ? 2 : 0) * n;
    wr[row - 1] += red[0][0];
    wr[n + row - 1] += red[1][0];
  }
}

// ---------------------------------------------------------------------------
// FP32 variant (mixed path).  On the reference grid k = dkr (i - dnk - 1/2) the
// energies are c u_i^2 with the odd integers u_i = 2 (i - dnk) - 1 and
// c = hbar^2 dkr^2 / (8 m), so the energy sums of the tables are exact integer
// forms: with the builder's (a, b, d),
//   eh: E = 2 (a - d) [ce (u_a + u_d) + ch (2 u_b + u_d - u_a)]
//   ee: E = 8 ce (a - d) (d - b),   hh: E = 8 ch (a - d) (d - b).
// x = E / (hbar g) is formed from these integers and split constants (head
// products exact), so the Lorentzian 1 / (1 + x^2) or the Gaussian exp(-x^2)
// carries no cancellation of the FP64 energies.  V^2 is scaled by its maximum per
// kind; the prefactors (2 g / (hbar g)^2 or (2 pi / hbar) / (sqrt(pi) hbar g)) and
// the V^2 scale are applied in FP64 to the block sums.  Per thread, the FP32 sums of
// one q2 row are added with compensation (Kahan); the block sums are FP64.

struct MbcConst {
  float aeh, ael, ahh, ahl;   // x_eh = 2 (a - d) (ae (u_a + u_d) + ah (2 u_b + u_d - u_a))
  float bee, bhh;             // x_ee = bee (a - d)(d - b), x_hh = bhh (a - d)(d - b)
  double peh, pee, phh;       // prefactor x V^2 scale per kind
};

__device__ __forceinline__ float split_head(double v) {
  // v rounded to 9 significant bits: its product with an integer of magnitude
  // below 2^15 is exact in FP32
  const float f = (float)v;
  return __uint_as_float(__float_as_uint(f) & 0xFFFF8000u);
}

template <bool LZ>
__device__ __forceinline__ float lor_or_gauss(float x) {
  const float x2 = x * x;
  if (LZ) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + x2));
    return r;
  }
  return __expf(-x2);
}

// Gaussian broadening: terms with |x| > MBC_XCUT (exp(-x^2) < 6e-19 of the
// largest) are left out; their FP32 value is below the sums' rounding.
constexpr float MBC_XCUT = 6.5f;

__device__ __forceinline__ int clamp_int(float v) {
  return (int)fminf(fmaxf(v, -1.0e6f), 1.0e6f);
}

// q in [lo, hi] with |2 (q - q2) (P q + Q)| <= MBC_XCUT (P != 0): the parabola
// 2 P (q - m)^2 - 2 P h^2 (roots q2 and -Q / P, midpoint m, half distance h) lies
// within +-X on [m - R+, m - R-] and [m + R-, m + R+], R+- = sqrt(h^2 +- X / (2P))
// (one interval when h^2 <= X / (2P)); bounds widened by 2; empty: lo > hi.
__device__ __forceinline__ void band_quad(float P, float Q, int q2, int lo, int hi, int& l1,
                                          int& h1, int& l2, int& h2) {
  if (P < 0.f) {
    P = -P;
    Q = -Q;
  }
  const float qs = -__fdividef(Q, P);   // band bounds carry a margin: fast divisions
  const float m = 0.5f * ((float)q2 + qs), h = 0.5f * (qs - (float)q2);
  const float t = __fdividef(MBC_XCUT, 2.f * P);
  const float Rp = sqrtf(h * h + t), hm = h * h - t;
  l1 = max(lo, clamp_int(floorf(m - Rp)) - 2);
  h2 = min(hi, clamp_int(ceilf(m + Rp)) + 2);
  if (hm <= 0.f) {
    h1 = h2;
    l2 = 1;
    h2 = 0;
    return;
  }
  const float Rm = sqrtf(hm);
  h1 = min(hi, clamp_int(ceilf(m - Rm)) + 2);
  l2 = max(lo, clamp_int(floorf(m + Rm)) - 2);
  if (l2 <= h1 + 1) {   // the two intervals touch: one
    h1 = max(h1, h2);
    l2 = 1;
    h2 = 0;
  }
}

// q1 range of |m (C + s q1)| <= MBC_XCUT (m > 0, s > 0), widened by 2
__device__ __forceinline__ void band_linear(float m, float C, float s, int& lo, int& hi) {
  const float c = __fdividef(MBC_XCUT, m), is = __fdividef(1.f, s);
  lo = max(lo, clamp_int(floorf((-c - C) * is)) - 2);
  hi = min(hi, clamp_int(ceilf((c - C) * is)) + 2);
}

template <bool LZ>
__global__ void __launch_bounds__(256) k_mbc_rates32(const WireDev* wires, int w_only,
                                                     const double2* nev, const double2* nhv,
                                                     const double* vs, double* wrate, int all) {
  const WireDev W = wires[w_only >= 0 ? w_only : blockIdx.y];
  const int n = W.nk;
  const int row = blockIdx.x + 1;
  if (row > n || !(all || (W.flags & SBE_F_EHS))) return;
  const bool lz = (W.flags & SBE_F_LORENTZ) != 0;
  if (lz != LZ) return;   // the other instantiation takes this wire
  const bool holes = blockIdx.z == 1;
  extern __shared__ float shf[];
  float* ne = shf;                 // [0, n], ne[0] = 0
  float* nh = shf + (n + 1);
  float* veh = shf + 2 * (n + 1);  // V_eh^2 / max, by k1 - k2 >= 0
  float* vxx = veh + n;            // V_ee^2 or V_hh^2 / max
  __shared__ MbcConst K;
  __shared__ double vmax[2][8];
  const double* vsw = vs + 3 * W.off_vec;
  const double* vx = vsw + (holes ? 2 : 1) * n;
  double m0 = 0.0, m1 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    m0 = fmax(m0, vsw[i] * vsw[i]);
    m1 = fmax(m1, vx[i] * vx[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    m0 = fmax(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, o));
  }
  if ((threadIdx.x & 31) == 0) {
    vmax[0][threadIdx.x >> 5] = m0;
    vmax[1][threadIdx.x >> 5] = m1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      vmax[0][0] = fmax(vmax[0][0], vmax[0][w]);
      vmax[1][0] = fmax(vmax[1][0], vmax[1][w]);
    }
    const double geh = (W.gam_e + W.gam_h) / 2.0;
    const double c0 = kHbar * kHbar * W.dkr * W.dkr / 8.0;
    const double ce = c0 / W.me, ch = c0 / W.mh;
    const double ae = ce / (kHbar * geh), ah = ch / (kHbar * geh);
    K.aeh = split_head(ae);
    K.ael = (float)(ae - (double)K.aeh);
    K.ahh = split_head(ah);
    K.ahl = (float)(ah - (double)K.ahh);
    K.bee = (float)(8.0 * ce / (kHbar * W.gam_e));
    K.bhh = (float)(8.0 * ch / (kHbar * W.gam_h));
    auto pref = [&](double g) {
      const double hg = kHbar * g;
      return lz ? 2.0 * g / (hg * hg) : kTwoPi / kHbar * (1.0 / (sqrt(kPi) * hg));
    };
    K.peh = pref(geh) * vmax[0][0];
    K.pee = pref(W.gam_e) * vmax[1][0];
    K.phh = pref(W.gam_h) * vmax[1][0];
  }
  __syncthreads();
  const double s0 = vmax[0][0] > 0.0 ? 1.0 / vmax[0][0] : 0.0;
  const double s1 = vmax[1][0] > 0.0 ? 1.0 / vmax[1][0] : 0.0;
  for (int i = threadIdx.x; i <= n; i += blockDim.x) {
    ne[i] = i == 0 ? 0.f : (float)fabs(nev[W.off_vec + i - 1].x);
    nh[i] = i == 0 ? 0.f : (float)fabs(nhv[W.off_vec + i - 1].x);
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    veh[i] = (float)(vsw[i] * vsw[i] * s0);
    vxx[i] = (float)(vx[i] * vx[i] * s1);
  }
  __syncthreads();
  const MbcConst k = K;
  const int dnk2 = 2 * W.dnk + 1;   // u_i = 2 i - dnk2 (builder index i)
  // x of the eh table at builder (a, b, d)
  auto x_eh = [&](int a, int b, int d) {
    const int ua = 2 * a - dnk2, ud = 2 * d - dnk2, ub = 2 * b - dnk2;
    const float i1 = (float)(ua + ud), i2 = (float)(2 * ub + ud - ua);
    const float s = (k.aeh * i1 + k.ahh * i2) + (k.ael * i1 + k.ahl * i2);
    return (float)(2 * (a - d)) * s;
  };
  // sums: win eh, win xx, wout eh, wout xx
  float part[4] = {0.f, 0.f, 0.f, 0.f}, accs[4] = {0.f, 0.f, 0.f, 0.f}, comp[4] = {0.f, 0.f, 0.f, 0.f};
  // warp w takes q2 = 2 + w, 2 + w + 8, ...; its lanes walk the q1 range in which
  // the term's indices are valid and its table value can be nonzero (q1, q2, the
  // row and the third index at least 2 for the one-lower table read, the third
  // index within [1, Nk], V^2 of a nonnegative index difference)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int r = row;
  if (r >= 2) {
    // eh band (Gaussian): x = 2 (a - d) S with S linear in b = q1 - 2 at fixed (a, d)
    const float ah_f = k.ahh + k.ahl, ae_f = k.aeh + k.ael;
    auto eh_band = [&](int a, int d, int& lo, int& hi) {
      if (LZ) return;
      const int ua = 2 * a - dnk2, ud = 2 * d - dnk2;
      const float C = ae_f * (float)(ua + ud) + ah_f * (float)(ud - ua - 2 * dnk2 - 8);
      band_linear((float)(2 * (a - d)), C, 4.f * ah_f, lo, hi);
    };
    // xx band (Gaussian): x = beta m (q - q1) with m > 0: |q - q1| <= w
    auto xx_band = [&](float beta, int m, int q, int& lo, int& hi) {
      if (LZ) return;
      const int w = clamp_int(__fdividef(MBC_XCUT, beta * (float)m)) + 2;
      lo = max(lo, q - w);
      hi = min(hi, q + w);
    };
    for (int q2 = 2 + warp; q2 <= n; q2 += nwarp) {
      if (!holes) {
        if (q2 < r) {
          const float ve = veh[r - q2], vx2 = vxx[r - q2], nq2 = ne[q2];
          // Win eh: (kp, k1) = (q1, q2), k1p = q1 + q2 - r
          int lo = max(2, r - q2 + 2), hi = n;
          eh_band(r - 2, q2 - 2, lo, hi);
          for (int q1 = lo + lane; q1 <= hi; q1 += 32)
            part[0] += ve * (1.f - nh[q1]) * nh[q1 + q2 - r] * nq2 *
                       lor_or_gauss<LZ>(x_eh(r - 2, q1 - 2, q2 - 2));
          // Win ee: (k2, k4) = (q1, q2), k30 = r + q1 - q2
          lo = 2;
          hi = n - r + q2;
          xx_band(k.bee, r - q2, q2, lo, hi);
          for (int q1 = lo + lane; q1 <= hi; q1 += 32)
            part[1] += vx2 * (1.f - ne[q1]) * ne[r + q1 - q2] * nq2 *
                       lor_or_gauss<LZ>(k.bee * (float)((r - q2) * (q2 - q1)));
        } else if (q2 > r) {
          const float ve = veh[q2 - r], vx2 = vxx[q2 - r], mq2 = 1.f - ne[q2];
          // Wout eh: (kp, k1) = (q1, q2), k1q = q1 + r - q2
          int lo = max(2, q2 - r + 2), hi = n;
          eh_band(q2 - 2, r - 2, lo, hi);
          for (int q1 = lo + lane; q1 <= hi; q1 += 32)
            part[2] += ve * mq2 * (1.f - nh[q1]) * nh[q1 + r - q2] *
                       lor_or_gauss<LZ>(x_eh(q2 - 2, q1 - 2, r - 2));
          // Wout ee: (k2, k4) = (q1, q2), k31 = q2 + q1 - r
          lo = 2;
          hi = n + r - q2;
          xx_band(k.bee, q2 - r, r, lo, hi);
          for (int q1 = lo + lane; q1 <= hi; q1 += 32)
            part[3] += vx2 * mq2 * (1.f - ne[q1]) * ne[q2 + q1 - r] *
                       lor_or_gauss<LZ>(k.bee * (float)((q2 - r) * (r - q1)));
        }
      } else {
        const float nq2 = ne[q2];
        // eh terms: x = 2 (q1 - q2) (P q1 + Q) is quadratic in q1; (Gaussian) the
        // loops walk the band of |x| <= MBC_XCUT and skip what lies beyond the cut
        const int ud = 2 * (q2 - 2) - dnk2, ub = 2 * (r - 2) - dnk2;
        int l1, h1, l2, h2;
        // Win eh (q1 > q2): (k, k1) = (q1, q2), k1p = r + q2 - q1
        l1 = q2 + 1;
        h1 = min(n, r + q2 - 2);
        l2 = 1;
        h2 = 0;
        if (!LZ)
          band_quad(2.f * (ae_f - ah_f),
                    (ae_f - ah_f) * (float)(-4 - dnk2) + ae_f * (float)ud + ah_f * (float)(2 * ub + ud),
                    q2, l1, h1, l1, h1, l2, h2);
#pragma unroll
        for (int j = 0; j < 2; ++j)
          for (int q1 = (j ? l2 : l1) + lane; q1 <= (j ? h2 : h1); q1 += 32) {
            const float x = x_eh(q1 - 2, r - 2, q2 - 2);
            if (!LZ && fabsf(x) > MBC_XCUT) continue;
            part[0] += veh[q1 - q2] * (1.f - ne[q1]) * nh[r + q2 - q1] * nq2 * lor_or_gauss<LZ>(x);
          }
        // Wout eh (q1 < q2): k1q = r + q1 - q2
        l1 = max(2, q2 - r + 2);
        h1 = q2 - 1;
        l2 = 1;
        h2 = 0;
        if (!LZ)
          band_quad(2.f * (ae_f + ah_f),
                    (ae_f + ah_f) * (float)(-4 - dnk2 + ud) + 4.f * ah_f * (float)(r - q2), q2,
                    l1, h1, l1, h1, l2, h2);
#pragma unroll
        for (int j = 0; j < 2; ++j)
          for (int q1 = (j ? l2 : l1) + lane; q1 <= (j ? h2 : h1); q1 += 32) {
            const int k1q = r + q1 - q2;
            const float x = x_eh(q1 - 2, k1q - 2, q2 - 2);
            if (!LZ && fabsf(x) > MBC_XCUT) continue;
            part[2] += veh[q2 - q1] * (1.f - ne[q1]) * (1.f - nh[k1q]) * nq2 * lor_or_gauss<LZ>(x);
          }
        if (q2 < r) {
          const float vx2 = vxx[r - q2], hq2 = nh[q2];
          // Win hh: (k2p, k4p) = (q1, q2), k3p = r + q1 - q2
          int lo = 2, hi = n - r + q2;
          xx_band(k.bhh, r - q2, q2, lo, hi);
          for (int q1 = lo + lane; q1 <= hi; q1 += 32)
            part[1] += vx2 * (1.f - nh[q1]) * nh[r + q1 - q2] * hq2 *
                       lor_or_gauss<LZ>(k.bhh * (float)((r - q2) * (q2 - q1)));
        } else if (q2 > r) {
          const float vx2 = vxx[q2 - r], mq2 = 1.f - nh[q2];
          // Wout hh: k3q = q2 + q1 - r
          int lo = 2, hi = n + r - q2;
          xx_band(k.bhh, q2 - r, r, lo, hi);
          for (int q1 = lo + lane; q1 <= hi; q1 += 32)
            part[3] += vx2 * mq2 * (1.f - nh[q1]) * nh[q2 + q1 - r] *
                       lor_or_gauss<LZ>(k.bhh * (float)((q2 - r) * (r - q1)));
        }
      }
      // per q2 row (at most Nk / 32 terms per lane and sum): compensated FP32
      // accumulation (an FP64 add per row and sum kept the FP64 pipe busy)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float y = part[j] - comp[j];
        const float t = accs[j] + y;
        comp[j] = (t - accs[j]) - y;
        accs[j] = t;
        part[j] = 0.f;
      }
    }
  }
  double acc[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) acc[j] = (double)accs[j] - (double)comp[j];
  __shared__ double red[4][256];
#pragma unroll
  for (int j = 0; j < 4; ++j) red[j][threadIdx.x] = acc[j];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
#pragma unroll
      for (int j = 0; j < 4; ++j) red[j][threadIdx.x] += red[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double px = holes ? k.phh : k.pee;
    double* wr = wrate + 4 * W.off_vec + (holes ? 2 : 0) * n;
    wr[row - 1] += k.peh * red[0][0] + px * red[1][0];
    wr[n + row - 1] += k.peh * red[2][0] + px * red[3][0];
  }
}

}  // namespace

// Adds the carrier-carrier in/out rates of every wire with EHs on (or of wire
// w_only; with all set, whatever its flags) to wrate, at the occupations in ne,
// nh and the screened V in vs.
void launch_mbc_rates(SbeCtx* c, int w_only, cudaStream_t s, bool all, bool fp32) {
  bool any = false;
  for (int w = 0; w < c->nw; ++w)
    if ((w_only < 0 || w == w_only) && (all || (c->wires[w].flags & SBE_F_EHS))) any = true;
  if (!any) return;
  const int nk = w_only >= 0 ? c->wires[w_only].nk : c->nk_max;
  if (fp32) {
    const size_t smf = sizeof(float) * (2 * (size_t)(nk + 1) + 2 * (size_t)nk);
    if (smf > 48 * 1024) {
      cudaFuncSetAttribute(k_mbc_rates32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smf);
      cudaFuncSetAttribute(k_mbc_rates32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smf);
    }
    // one instantiation per broadening; each skips the other's wires
    bool gauss = false, lor = false;
    for (int w = 0; w < c->nw; ++w)
      if (w_only < 0 || w == w_only) (c->wires[w].flags & SBE_F_LORENTZ ? lor : gauss) = true;
    const dim3 grid(nk, w_only >= 0 ? 1 : c->nw, 2);
    if (gauss)
      k_mbc_rates32<false><<<grid, 256, smf, s>>>(c->d_wires, w_only, c->ne, c->nh, c->vs,
                                                   c->wrate, all ? 1 : 0);
    if (lor)
      k_mbc_rates32<true><<<grid, 256, smf, s>>>(c->d_wires, w_only, c->ne, c->nh, c->vs,
                                                  c->wrate, all ? 1 : 0);
    return;
  }
  const size_t sm = sizeof(double) * (2 * (size_t)(nk + 1) + 3 * (size_t)nk);
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_mbc_rates64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_mbc_rates64<<<dim3(nk, w_only >= 0 ? 1 : c->nw, 2), 256, sm, s>>>(
      c->d_wires, w_only, c->ne, c->nh, c->vs, c->Ee, c->Eh, c->wrate, all ? 1 : 0);
}

}  // namespace sbe
