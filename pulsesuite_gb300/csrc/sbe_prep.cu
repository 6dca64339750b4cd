// Per-step preparation of every wire: occupations, screening, diagonal and
// off-diagonal dephasing, and the Hartree-Fock Hamiltonians (FP64).
#include "sbe_ctx.cuh"
#include "fp_bits.cuh"

namespace sbe {

// ---------------------------------------------------------------------------
// SBEs.py:5200-5204 (ne, nh = diag C, diag D) and coulomb.py:1172-1230
// (CalcScreenedArrays / Eps1D).  On the reference grid every Coulomb table is a
// function of k1-k2 only: V0[k1,k2] = v0(k1-k2) for k1 >= k2 and 0 above the
// diagonal (kkp < 0 is skipped), E1D[k1,k2] = eps(|k1-k2|).  One block per wire
// forms ne, nh, n1D and the screened vs(d) = v0(d)/eps(d).
__global__ void k_extract_diag(const WireDev* wires, const double2* C, const double2* D,
                               double2* ne, double2* nh) {
  const WireDev W = wires[blockIdx.x];
  const int nk = W.nk;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    ne[W.off_vec + k] = C[W.off_mat + (long long)k * nk + k];
    nh[W.off_vec + k] = D[W.off_mat + (long long)k * nk + k];
  }
}

void launch_extract_diag(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s) {
  k_extract_diag<<<c->nw, 256, 0, s>>>(c->d_wires, C, D, c->ne, c->nh);
}

__global__ void k_screen(const WireDev* wires, int w_only, const double* v0, const double* chi,
                         const double* qeh, const double2* ne, const double2* nh, double* eps,
                         double* vs) {
  const WireDev W = wires[w_only >= 0 ? w_only : blockIdx.x];
  const int nk = W.nk;
  __shared__ double red[256];
  double s = 0.0;
  for (int k = threadIdx.x; k < nk; k += blockDim.x)
    s += ne[W.off_vec + k].x + nh[W.off_vec + k].x;
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  double n1d = red[0] / 2.0 / W.L;
  n1d = fmin(n1d, W.nmax);
  const bool screened = (W.flags & SBE_F_SCREENED) != 0;
  for (int d = threadIdx.x; d < nk; d += blockDim.x) {
    double e = 1.0;
    if (screened) {
      double qe = qeh[2 * W.off_vec + d], qh = qeh[2 * W.off_vec + nk + d];
      double ce = chi[2 * W.off_vec + d], chh = chi[2 * W.off_vec + nk + d];
      e = 1.0 - ce * 2 * log(fabs((qe - kPi * n1d) / (qe + n1d))) -
          chh * 2 * log(fabs((qh - kPi * n1d) / (qh + n1d)));
    }
    eps[W.off_vec + d] = e;
    for (int n = 0; n < 3; ++n)
      vs[3 * W.off_vec + n * nk + d] = v0[3 * W.off_vec + n * nk + d] / e;
  }
}

void launch_screen(SbeCtx* c, int w_only, cudaStream_t s) {
  k_screen<<<w_only >= 0 ? 1 : c->nw, 256, 0, s>>>(c->d_wires, w_only, c->v0, c->chi, c->qeh,
                                                   c->ne, c->nh, c->eps, c->vs);
}

void launch_prep_scalar(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s) {
  launch_extract_diag(c, C, D, s);
  launch_screen(c, -1, s);
  launch_spont(c, -1, s);   // Recomb: SBEs.py:5203-5226
}

// Expand to the reference's (Nk, Nk, 3) VC and (Nk, Nk) E1D of wire w.
__global__ void k_expand_vc(const WireDev* wires, int w, const double* vs, const double* eps,
                            double* VC, double* E1D) {
  const WireDev W = wires[w];
  int k2 = blockIdx.x * blockDim.x + threadIdx.x;
  int k1 = blockIdx.y;
  if (k1 >= W.nk || k2 >= W.nk) return;
  int d = k1 - k2;
  long long o = (long long)k1 * W.nk + k2;
  for (int n = 0; n < 3; ++n)
    VC[3 * o + n] = d >= 0 ? vs[3 * W.off_vec + n * W.nk + d] : 0.0;
  E1D[o] = eps[W.off_vec + (d >= 0 ? d : -d)];
}

void launch_expand_vc(SbeCtx* c, int w, double* VC, double* E1D, cudaStream_t s) {
  int nk = c->wires[w].nk;
  k_expand_vc<<<dim3((nk + 127) / 128, nk), 128, 0, s>>>(c->d_wires, w, c->vs, c->eps, VC, E1D);
}

// ---------------------------------------------------------------------------
// dephasing.py:29-103 (_CalcGammaE_jit/_CalcGammaH_jit) with the index maps of
// InitializeDephasing and Vxx2 (V[round(|k/dk|), 0]^2, dephasing.py:362-378).
// One warp per (wire, k), lanes over q.
__device__ inline double occ_ext(const double2* n, int idx, int nk, bool* ok) {
  // extended array of the reference: index idx+1 in [1, nk] is valid
  if (idx < 0 || idx >= nk) { *ok = false; return 0.0; }
  *ok = true;
  return n[idx].x;
}

__global__ void k_gamma(const WireDev* wires, int w_only, const double2* ne, const double2* nh,
                        const double* vs, const int* iq, const int* maps, const double* xeh,
                        double* gamE, double* gamH) {
  int wi = (w_only >= 0) ? w_only : blockIdx.y;
  const WireDev W = wires[wi];
  const int nk = W.nk;
  int k = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int lane = threadIdx.x & 31;
  if (k >= nk) return;
  if (!(W.flags & SBE_F_DIAGDPH)) {
    if (lane == 0) {
      gamE[W.off_vec + k] = W.gam_e;
      gamH[W.off_vec + k] = W.gam_h;
    }
    return;
  }
  const double2* pe = ne + W.off_vec;
  const double2* ph = nh + W.off_vec;
  const long long st = (long long)nk * nk;
  const int* m = maps + 6 * W.off_mat + (long long)k * nk;
  const double* v = vs + 3 * W.off_vec;
  const double* xe = xeh + 2 * W.off_vec;
  const double* xh = xe + nk;
  const double pih = kPi / kHbar;
  double ge = 0.0, gh = 0.0;
  for (int q = lane; q < nk; q += 32) {
    int iqq = iq[W.off_vec + q];
    double veh = v[0 * nk + iqq], vee = v[1 * nk + iqq], vhh = v[2 * nk + iqq];
    double veh2 = veh * veh, vee2 = vee * vee, vhh2 = vhh * vhh;
    bool ok, ok1, ok2, ok3;
    // electrons
    double a = occ_ext(pe, m[0 * st + q], nk, &ok);
    if (ok) ge += pih * vee2 * a * (1.0 - a) * fabs(xe[q]);
    double n1 = occ_ext(ph, m[3 * st + q], nk, &ok1);   // k1p_m_q
    double n2 = occ_ext(ph, m[2 * st + q], nk, &ok2);   // k1p
    double n3 = occ_ext(pe, m[1 * st + q], nk, &ok3);   // k_m_q
    if (ok1 && ok2 && ok3)
      ge += pih * veh2 * (n1 * (1.0 - n2) * n3 + (1.0 - n1) * n2 * (1.0 - n3)) * fabs(xh[q]);
    // holes
    double b = occ_ext(ph, m[0 * st + q], nk, &ok);
    if (ok) gh += pih * vhh2 * b * (1.0 - b) * fabs(xh[q]);
    double e1 = occ_ext(pe, m[5 * st + q], nk, &ok1);   // k1_m_q
    double e2 = occ_ext(pe, m[4 * st + q], nk, &ok2);   // k1
    double h3 = occ_ext(ph, m[1 * st + q], nk, &ok3);   // k_m_q
    if (ok1 && ok2 && ok3)
      gh += pih * veh2 * (e1 * (1.0 - e2) * h3 + (1.0 - e1) * e2 * (1.0 - h3)) * fabs(xe[q]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ge += __shfl_down_sync(0xffffffffu, ge, o);
    gh += __shfl_down_sync(0xffffffffu, gh, o);
  }
  if (lane == 0) {
    gamE[W.off_vec + k] = ge;
    gamH[W.off_vec + k] = gh;
  }
}

void launch_gamma(SbeCtx* c, int w_only, cudaStream_t s) {
  int wpb = 8;
  dim3 g((c->nk_max + wpb - 1) / wpb, w_only >= 0 ? 1 : c->nw);
  k_gamma<<<g, 32 * wpb, 0, s>>>(c->d_wires, w_only, c->ne, c->nh, c->vs, c->iq, c->maps,
                                 c->xeh, c->gamE, c->gamH);
}

// ---------------------------------------------------------------------------
// dephasing.py:227-317 (_CalcOffDiagDeph_E2_jit / _H2_jit): D[q+Nk][k] for one
// carrier species "a" (electrons for De, holes for Dh) against itself and the
// other species "b".  FP64, literal energy differences from the Ee/Eh arrays.
// g3 = [gam_eh, gam_e, gam_h]: De uses (g0, g2), Dh uses (g1, g2) (quirk kept).
__global__ void k_offdiag_D64(const WireDev* wires, int w_only, const double2* ne,
                              const double2* nh, const double* Ee, const double* Eh,
                              const double* vs, double g0, double g1, double g2, int use_g,
                              double* De, double* Dh) {
  int wi = (w_only >= 0) ? w_only : blockIdx.z;
  const WireDev W = wires[wi];
  const int nk = W.nk;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  int qi = blockIdx.y >> 1;          // 0 .. 2nk
  int which = blockIdx.y & 1;        // 0 -> De, 1 -> Dh
  if (qi > 2 * nk || k >= nk) return;
  int q = qi - nk;
  double ga = use_g ? (which == 0 ? g0 : g1) : (which == 0 ? W.gam_eh : W.gam_e);
  double gab = use_g ? g2 : W.gam_h;
  const double2* na = (which == 0 ? ne : nh) + W.off_vec;
  const double2* nb = (which == 0 ? nh : ne) + W.off_vec;
  const double* Ea = (which == 0 ? Ee : Eh) + W.off_vec;
  const double* Eb = (which == 0 ? Eh : Ee) + W.off_vec;
  const double* v = vs + 3 * W.off_vec;
  int aq = q < 0 ? -q : q;
  double vaa = 0.0, vab = 0.0;
  if (aq >= 1 && aq < nk) {
    double x = v[(which == 0 ? 1 : 2) * nk + aq];
    double y = v[0 * nk + aq];
    vaa = x * x;
    vab = y * y;
  }
  double acc = 0.0;
  if (k + q >= 0 && k + q < nk) {
    double nak = hypot(na[k].x, na[k].y);
    double bb = kHbar * ga, b2 = kHbar * gab;
    if (vaa != 0.0) {
      int plo = max(q + 1, 0), phi = min(q + nk - 1, nk - 1);
      for (int p = plo; p <= phi; ++p) {
        double Ed = Ea[k + q] + Ea[p - q] - Ea[p] - Ea[k];
        double npq = hypot(na[p - q].x, na[p - q].y);
        double np_ = hypot(na[p].x, na[p].y);
        double lr = (bb / kPi) / (Ed * Ed + bb * bb);
        acc += vaa * lr * (npq * (1.0 - np_) * (1.0 - nak) + (1.0 - npq) * np_ * nak);
      }
    }
    if (vab != 0.0) {
      int plo = max(0, -q), phi = min(nk - 1, nk - 1 - q);
      for (int p = plo; p <= phi; ++p) {
        double Ed = Ea[k + q] + Eb[p + q] - Eb[p] - Ea[k];
        double npq = hypot(nb[p + q].x, nb[p + q].y);
        double np_ = hypot(nb[p].x, nb[p].y);
        double lr = (b2 / kPi) / (Ed * Ed + b2 * b2);
        acc += vab * lr * (npq * (1.0 - np_) * (1.0 - nak) + (1.0 - npq) * np_ * nak);
      }
    }
  }
  double* D = (which == 0 ? De : Dh) + W.off_dd;
  D[(long long)qi * nk + k] = acc * kPi / kHbar;
}

// FP32 version of the off-diagonal dephasing sums for the mixed-precision path.
// On the reference grid (parabolic bands, kr = dkr (j - j0), j0 = dnk + 1/2)
// the energy differences are exact integer multiples of one constant:
//   a-a:  E = 2 c_a dkr^2 q (k - p + q)
//   a-b:  E = dkr^2 q [c_a (2k - 2j0 + q) + c_b (2p - 2j0 + q)]
// so u = E/(hbar g) is formed without cancellation (the a-b constants are split
// into an 11-bit head, whose products with the integers |2k + c| < 2^12 are
// exact in FP32, and a tail).  Lorentz(E, b) = (1/(pi b)) / (1 + u^2).  The a-a
// kernel depends on k - p only, so it is tabulated per q in shared memory.  One
// block per (k tile, q, wire x {De, Dh}); the (1 - n_k) / n_k split of the
// occupation product makes the p-sums two dot products per thread.
__device__ inline void split12(double v, float* hi, float* lo) {
  int ex;
  double m = frexp(v, &ex);                 // v = m 2^ex, 0.5 <= |m| < 1
  double h = ldexp(rint(ldexp(m, 11)), ex - 11);
  *hi = (float)h;
  *lo = (float)(v - h);
}

__global__ void k_occf(const WireDev* wires, const double2* ne, const double2* nh, float* occf) {
  const WireDev& W = wires[blockIdx.y];
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= W.nk) return;
  occf[2 * W.off_vec + k] = (float)hypot(ne[W.off_vec + k].x, ne[W.off_vec + k].y);
  occf[2 * W.off_vec + W.nk + k] = (float)hypot(nh[W.off_vec + k].x, nh[W.off_vec + k].y);
}

// One block per (q >= 0, species, wire) and up to 512 k; each thread sums four
// consecutive k, so that the per-p shared-memory loads (the Lorentzian window and
// the paired occupation weights, read as one float2 broadcast) serve four outputs.
//
// The rows -q come from the sums of row q.  With p' = p - q (a-a) or p' = p + q
// (a-b) the term (-q, k + q, p') has the Lorentzian argument -u(q, k, p) and the
// two occupation weights of (q, k, p) swapped, over the same p range, except
// that the a-a range of row -q also holds p' = 0 (p = q), which row q leaves out
// (p - q >= 1 in the reference loops).  So
//   sa(-q, k + q) = sb(q, k) [+ the a-a term p = q],  sb(-q, k + q) = sa(q, k) [+ ..]
// and a block writes D[q][k] and D[-q][k + q] for every k with k + q < Nk, and
// the zeros of both rows elsewhere; the Lorentzian sums are formed once.
__global__ void __launch_bounds__(128) k_offdiag_D32(const WireDev* wires, const int* wl,
                                                     const float* occf,
                                                     const float* dconst, const float* dpre,
                                                     double* De, double* Dh) {
  const int wi = wl[blockIdx.z >> 1], which = blockIdx.z & 1;   // 0 De, 1 Dh
  const WireDev& W = wires[wi];
  const int nk = W.nk;
  const int q = blockIdx.y;   // 0 .. nk; row -q from the same sums
  if (q > nk) return;
  extern __shared__ float sh[];
  float* na = sh;                                        // |n_a|
  float* nb = na + nk;                                   // |n_b|
  float* Ltab = nb + nk;                                 // 2nk entries: m - mlo
  float2* wa = reinterpret_cast<float2*>(Ltab + 2 * nk); // (Aa, Ba) per p (a-a)
  float2* wb = wa + nk;                                  // (Ab, Bb) per p (a-b)
  // |n_e|, |n_h| as FP32 (formed once per step by k_occf)
  const float* pa = occf + 2 * W.off_vec + (which == 0 ? 0 : nk);
  const float* pb = occf + 2 * W.off_vec + (which == 0 ? nk : 0);
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    na[i] = pa[i];
    nb[i] = pb[i];
  }
  // per-(wire, species) constants and per-q prefactors (k_deph_consts)
  const float* cw = dconst + (long long)(2 * wi + which) * 8;
  const float alpha = cw[0] * (float)q;
  const float bah = cw[1], bal = cw[2], bbh = cw[3], bbl = cw[4];
  const float* pq = dpre + 2 * (2 * W.off_vec + (long long)which * nk) + 0;
  const int aq = q < 0 ? -q : q;
  const float vaa = (aq >= 1 && aq < nk) ? pq[2 * aq] : 0.f;
  const float vab = (aq >= 1 && aq < nk) ? pq[2 * aq + 1] : 0.f;
  const int mlo = -nk + 1 + q;
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * nk; i += blockDim.x) {
    float u = alpha * (float)(mlo + i);
    Ltab[i] = 1.0f / (1.0f + u * u);
  }
  for (int p = threadIdx.x; p < nk; p += blockDim.x) {
    int pm = p - q, pp = p + q;
    bool okm = pm >= 0 && pm < nk, okp = pp >= 0 && pp < nk;
    float a_pm = okm ? na[pm] : 0.f, b_pp = okp ? nb[pp] : 0.f;
    wa[p] = make_float2(okm ? a_pm * (1.f - na[p]) : 0.f, okm ? (1.f - a_pm) * na[p] : 0.f);
    wb[p] = make_float2(okp ? b_pp * (1.f - nb[p]) : 0.f, okp ? (1.f - b_pp) * nb[p] : 0.f);
  }
  __syncthreads();
  double* D = (which == 0 ? De : Dh) + W.off_dd;
  double* Dp = D + (long long)(nk + q) * nk;   // row q
  double* Dm = D + (long long)(nk - q) * nk;   // row -q
  // the a-a term p = q of row -q (absent from row q): L(alpha q k) weights
  const float n0a = na[0], nqa = (q < nk) ? na[q] : 0.f;
  for (int k0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4; k0 < nk;
       k0 += gridDim.x * blockDim.x * 4) {
    float sa[4] = {0.f, 0.f, 0.f, 0.f}, sb[4] = {0.f, 0.f, 0.f, 0.f};
    if (vaa != 0.f) {
      const int plo = max(q + 1, 0), phi = min(q + nk - 1, nk - 1);
      // L index of (k, p) is k - p + nk - 1; the window holds k0 .. k0 + 3 at this p
      float l[4];
      const int i0 = k0 - plo + nk - 1;
#pragma unroll
      for (int j = 0; j < 4; ++j) l[j] = (i0 + j < 2 * nk) ? Ltab[i0 + j] : 0.f;
      for (int p = plo; p <= phi; ++p) {
        const float2 w2 = wa[p];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          sa[j] = fmaf(l[j], w2.x, sa[j]);
          sb[j] = fmaf(l[j], w2.y, sb[j]);
        }
        // next p: index - 1
        const int in = i0 - (p + 1 - plo);
#pragma unroll
        for (int j = 3; j > 0; --j) l[j] = l[j - 1];
        l[0] = (in >= 0) ? Ltab[in] : 0.f;
      }
    }
    float ta[4], tb[4];   // a-b sums
#pragma unroll
    for (int j = 0; j < 4; ++j) ta[j] = tb[j] = 0.f;
    if (vab != 0.f) {
      const int plo = max(0, -q), phi = min(nk - 1, nk - 1 - q);
      const int c = -2 * W.dnk - 1 + q;
      float ka[4], kal[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float fk = (float)(2 * (k0 + j) + c);
        ka[j] = bah * fk;   // exact head product
        kal[j] = bal * fk;  // tail
      }
      const float fq = (float)q;
      float fp = (float)(2 * plo + c);   // exact small integers, stepped by 2
      for (int p = plo; p <= phi; ++p, fp += 2.0f) {
        const float2 w2 = wb[p];
        const float hb = bbh * fp;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float sv = (ka[j] + hb) + fmaf(bbl, fp, kal[j]);
          const float u = fq * sv;
          float L;   // 1/(1+u^2) >= 1e-38: the approximate reciprocal (~1 ulp) suffices
          asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(L) : "f"(fmaf(u, u, 1.0f)));
          ta[j] = fmaf(L, w2.x, ta[j]);
          tb[j] = fmaf(L, w2.y, tb[j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = k0 + j;
      if (k >= nk) continue;
      if (k + q >= nk) {
        // row q outside the band; row -q at k' = k - (nk - q) < q is zero too
        Dp[k] = 0.0;
        if (q > 0) Dm[k - (nk - q)] = 0.0;
        continue;
      }
      const float nak = na[k];
      const float vq = vaa * ((1.f - nak) * sa[j] + nak * sb[j]) +
                       vab * ((1.f - nak) * ta[j] + nak * tb[j]);
      Dp[k] = f32_to_f64(vq);
      if (q > 0) {
        // row -q at k + q: swapped sums plus the a-a term p = q
        const float lq = Ltab[k + nk - 1 - q];   // L(alpha q k)
        const float xa = sb[j] + lq * ((1.f - n0a) * nqa);
        const float xb = sa[j] + lq * (n0a * (1.f - nqa));
        const float nk2 = na[k + q];
        const float vm = vaa * ((1.f - nk2) * xa + nk2 * xb) +
                         vab * ((1.f - nk2) * tb[j] + nk2 * ta[j]);
        Dm[k + q] = f32_to_f64(vm);
      }
    }
  }
}

// The same sums for a group of NW wires that share their Lorentzian factors (same
// Nk, masses, grid and rates): each Lorentzian is formed once and applied to every
// wire's occupation weights, which carry the per-wire prefactors V_aa(q)^2 /
// (hbar b_aa), V_ab(q)^2 / (hbar b_ab) (folded in, so one pair of sums per wire:
// X = (vaa sa + vab ta, vaa sb + vab tb)).  Each thread sums KPT consecutive k for
// all NW wires, so that every shared-memory weight load (32 p at a time, [p][wire]
// as float2, read as float4) feeds 2 KPT FMAs; the a-a Lorentzian window slides in
// registers.  Rows q and -q as in k_offdiag_D32.  grid (Nk / (128 KPT), Nk + 1, species).
// Packed FP32 pairs (PTX f32x2, sm_100 and later): one fma.rn.f32x2 forms two
// IEEE FP32 fused multiply-adds (each rounded as fmaf) from one issue slot.
__device__ __forceinline__ unsigned long long f2_splat(float a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a));
  return r;
}
__device__ __forceinline__ void f2_fma(unsigned long long& d, unsigned long long a,
                                       unsigned long long b) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(d) : "l"(a), "l"(b));
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long a) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a));
  return r;
}

template <int NW, int KPT>
__global__ void __launch_bounds__(128, 2) k_offdiag_D32g(const WireDev* wires, const int* wl,
                                                      int nwl, const float* occf,
                                                      const float* dconst, const float* dpre,
                                                      double* De, double* Dh) {
  constexpr int PC = 32;   // p per shared-memory chunk
  const int which = blockIdx.z;
  const WireDev& W0 = wires[wl[0]];
  const int nk = W0.nk;
  const int q = blockIdx.y;
  if (q > nk) return;
  extern __shared__ __align__(16) float sh[];
  float2* ws = reinterpret_cast<float2*>(sh);   // [PC][NW]
  float* Ltab = sh + 2 * PC * NW;               // 2nk entries: m - mlo
  __shared__ float svaa[NW], svab[NW], sn0[NW], snq[NW];
  __shared__ int soa[NW], sob[NW];              // occupation offsets of species a, b
  const int tid = threadIdx.x;
  const float* cw = dconst + (long long)(2 * wl[0] + which) * 8;
  const float alpha = cw[0] * (float)q;
  const float bah = cw[1], bal = cw[2], bbh = cw[3], bbl = cw[4];
  const int mlo = -nk + 1 + q;
  for (int i = tid; i < 2 * nk; i += blockDim.x) {
    const float u = alpha * (float)(mlo + i);
    Ltab[i] = 1.0f / (1.0f + u * u);
  }
  const bool inq = q >= 1 && q < nk;   // V(q) vanishes at q = 0 and |q| = Nk
  if (tid < NW) {
    float vaa = 0.f, vab = 0.f, n0 = 0.f, nq = 0.f;
    int oa = 0, ob = 0;
    if (tid < nwl) {
      const WireDev& W = wires[wl[tid]];
      oa = (int)(2 * W.off_vec + (which == 0 ? 0 : nk));
      ob = (int)(2 * W.off_vec + (which == 0 ? nk : 0));
      const float* pq = dpre + 2 * (2 * W.off_vec + (long long)which * nk);
      if (inq) {
        vaa = pq[2 * q];
        vab = pq[2 * q + 1];
      }
      n0 = occf[oa];
      nq = q < nk ? occf[oa + q] : 0.f;
    }
    svaa[tid] = vaa;
    svab[tid] = vab;
    sn0[tid] = n0;
    snq[tid] = nq;
    soa[tid] = oa;
    sob[tid] = ob;
  }
  const int k0 = (blockIdx.x * blockDim.x + tid) * KPT;   // this thread's first k
  // sums (x, y) of wire w at k0 + j as one packed FP32 pair; the weights of a
  // wire are the pair (x, y) in shared memory, so one f32x2 FMA updates both
  unsigned long long acc[KPT][NW];
#pragma unroll
  for (int j = 0; j < KPT; ++j)
#pragma unroll
    for (int w = 0; w < NW; ++w) acc[j][w] = 0ull;
  if (inq) {
    // a-a: p in [q + 1, Nk - 1], Lorentzian of alpha q (k - p + q) from the table;
    // index of (k, p) is k - p + Nk - 1: the window holds k0 .. k0 + KPT - 1
    float l[KPT];
    {
      const int i0 = k0 - (q + 1) + nk - 1;
#pragma unroll
      for (int j = 0; j < KPT; ++j) l[j] = 0.f;
      __syncthreads();   // the table is complete
#pragma unroll
      for (int j = 0; j < KPT; ++j)
        if (i0 + j >= 0 && i0 + j < 2 * nk) l[j] = Ltab[i0 + j];
    }
    for (int p0 = q + 1; p0 < nk; p0 += PC) {
      __syncthreads();
      for (int i = tid; i < PC * NW; i += blockDim.x) {
        const int pp = i / NW, w = i % NW, p = p0 + pp;
        float2 v = make_float2(0.f, 0.f);
        if (p < nk && w < nwl) {
          const float* na = occf + soa[w];
          const float npm = na[p - q], np_ = na[p], f = svaa[w];
          v = make_float2(f * (npm * (1.f - np_)), f * ((1.f - npm) * np_));
        }
        ws[i] = v;
      }
      __syncthreads();
      const int pend = min(PC, nk - p0);
      for (int pp = 0; pp < pend; ++pp) {
        const ulonglong2* w4 = reinterpret_cast<const ulonglong2*>(ws + pp * NW);
        unsigned long long ll[KPT];
#pragma unroll
        for (int j = 0; j < KPT; ++j) ll[j] = f2_splat(l[j]);
#pragma unroll
        for (int w2 = 0; w2 < NW / 2; ++w2) {
          const ulonglong2 v = w4[w2];
#pragma unroll
          for (int j = 0; j < KPT; ++j) {
            f2_fma(acc[j][2 * w2], ll[j], v.x);
            f2_fma(acc[j][2 * w2 + 1], ll[j], v.y);
          }
        }
        // next p: every index - 1
#pragma unroll
        for (int j = KPT - 1; j > 0; --j) l[j] = l[j - 1];
        const int in = k0 - (p0 + pp + 1) + nk - 1;
        l[0] = (in >= 0 && in < 2 * nk) ? Ltab[in] : 0.f;
      }
    }
    // a-b: p in [0, Nk - 1 - q], u = q (A (2k + c) + B (2p + c)) with exact heads
    const int c = -2 * W0.dnk - 1 + q;
    float ka[KPT], kal[KPT];
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const float fk = (float)(2 * (k0 + j) + c);
      ka[j] = bah * fk;   // exact head product
      kal[j] = bal * fk;  // tail
    }
    const float fq = (float)q;
    const int phi = nk - 1 - q;
    for (int p0 = 0; p0 <= phi; p0 += PC) {
      __syncthreads();
      for (int i = tid; i < PC * NW; i += blockDim.x) {
        const int pp = i / NW, w = i % NW, p = p0 + pp;
        float2 v = make_float2(0.f, 0.f);
        if (p <= phi && w < nwl) {
          const float* nb = occf + sob[w];
          const float npq = nb[p + q], np_ = nb[p], f = svab[w];
          v = make_float2(f * (npq * (1.f - np_)), f * ((1.f - npq) * np_));
        }
        ws[i] = v;
      }
      __syncthreads();
      const int pend = min(PC, phi + 1 - p0);
      float fp = (float)(2 * p0 + c);   // exact small integers, stepped by 2
      for (int pp = 0; pp < pend; ++pp, fp += 2.0f) {
        const float hb = bbh * fp, tb = bbl * fp;
        float L[KPT];
#pragma unroll
        for (int j = 0; j < KPT; ++j) {
          const float sv = (ka[j] + hb) + (kal[j] + tb);
          const float u = fq * sv;
          // 1/(1+u^2) >= 1e-38: the approximate reciprocal (~1 ulp) suffices
          asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(L[j]) : "f"(fmaf(u, u, 1.0f)));
        }
        const ulonglong2* w4 = reinterpret_cast<const ulonglong2*>(ws + pp * NW);
        unsigned long long ll[KPT];
#pragma unroll
        for (int j = 0; j < KPT; ++j) ll[j] = f2_splat(L[j]);
#pragma unroll
        for (int w2 = 0; w2 < NW / 2; ++w2) {
          const ulonglong2 v = w4[w2];
#pragma unroll
          for (int j = 0; j < KPT; ++j) {
            f2_fma(acc[j][2 * w2], ll[j], v.x);
            f2_fma(acc[j][2 * w2 + 1], ll[j], v.y);
          }
        }
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const int k = k0 + j;
    if (k >= nk) break;
    const float lq = q > 0 ? Ltab[k + nk - 1 - q] : 0.f;   // L(alpha q k): a-a term p = q of row -q
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      if (w >= nwl) break;
      const WireDev& W = wires[wl[w]];
      double* D = (which == 0 ? De : Dh) + W.off_dd;
      double* Dp = D + (long long)(nk + q) * nk;   // row q
      double* Dm = D + (long long)(nk - q) * nk;   // row -q
      const float* na = occf + soa[w];
      if (k + q >= nk) {
        Dp[k] = 0.0;
        if (q > 0) Dm[k - (nk - q)] = 0.0;
        continue;
      }
      const float nak = na[k];
      const float2 sxy = f2_unpack(acc[j][w]);
      Dp[k] = f32_to_f64((1.f - nak) * sxy.x + nak * sxy.y);
      if (q > 0) {
        const float f = svaa[w] * lq;
        const float xa = sxy.y + f * ((1.f - sn0[w]) * snq[w]);
        const float xb = sxy.x + f * (sn0[w] * (1.f - snq[w]));
        const float nk2 = na[k + q];
        Dm[k + q] = f32_to_f64((1.f - nk2) * xa + nk2 * xb);
      }
    }
  }
}

// Constants of k_offdiag_D32 (FP64, once per step): per (wire, species)
// [2 c_a dkr^2 / b_aa, head/tail of c_a dkr^2 / b_ab, head/tail of c_b dkr^2 / b_ab]
// and per |q| the prefactors V_aa(q)^2 / (hbar b_aa) and V_ab(q)^2 / (hbar b_ab)
// (D = (pi/hbar) V^2 Lorentz = V^2 / (hbar b) / (1 + u^2)).
__global__ void k_deph_consts(const WireDev* wires, const double* vs, float* dconst, float* dpre) {
  const int wi = blockIdx.y >> 1, which = blockIdx.y & 1;
  const WireDev& W = wires[wi];
  const int nk = W.nk;
  const double ma = which == 0 ? W.me : W.mh, mbm = which == 0 ? W.mh : W.me;
  const double ca = kHbar * kHbar / (2.0 * ma), cb = kHbar * kHbar / (2.0 * mbm);
  const double dk2 = W.dkr * W.dkr;
  const double g_aa = which == 0 ? W.gam_eh : W.gam_e;   // quirk: De uses gam_eh, Dh gam_e
  const double b_aa = kHbar * g_aa, b_ab = kHbar * W.gam_h;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    float* cw = dconst + (long long)(2 * wi + which) * 8;
    cw[0] = (float)(2.0 * ca * dk2 / b_aa);
    split12(ca * dk2 / b_ab, &cw[1], &cw[2]);
    split12(cb * dk2 / b_ab, &cw[3], &cw[4]);
  }
  const double* v = vs + 3 * W.off_vec;
  float* pq = dpre + 2 * (2 * W.off_vec + (long long)which * nk);
  for (int aq = blockIdx.x * blockDim.x + threadIdx.x; aq < nk; aq += gridDim.x * blockDim.x) {
    double x = v[(which == 0 ? 1 : 2) * nk + aq], y = v[aq];
    pq[2 * aq] = (float)(x * x / (kHbar * b_aa));
    pq[2 * aq + 1] = (float)(y * y / (kHbar * b_ab));
  }
}

void launch_offdiag_D(SbeCtx* c, int w_only, const double* g3, bool fp32, cudaStream_t s) {
  if (fp32 && w_only < 0 && !g3) {
    k_occf<<<dim3((c->nk_max + 127) / 128, c->nw), 128, 0, s>>>(c->d_wires, c->ne, c->nh,
                                                                 c->occf);
    k_deph_consts<<<dim3((c->nk_max + 127) / 128, 2 * c->nw), 128, 0, s>>>(c->d_wires, c->vs,
                                                                          c->dconst, c->dpre);
    // groups of 4 or more wires share the Lorentzian factors (chunks of up to 16
    // wires); the other wires take the per-wire kernel, one launch each
    for (const auto& g : c->dgroups) {
      const int gk = c->wires[c->dwl_host[g.first]].nk;
      if (g.second < 4) {
        const size_t sm1 = sizeof(float) * 8 * (size_t)gk;
        for (int i = 0; i < g.second; ++i)
          k_offdiag_D32<<<dim3((gk + 511) / 512, gk + 1, 2), 128, sm1, s>>>(
              c->d_wires, c->dwl + g.first + i, c->occf, c->dconst, c->dpre, c->De, c->Dh);
        continue;
      }
      const dim3 grid((gk + 511) / 512, gk + 1, 2);   // 128 threads x 4 k
      for (int o = 0; o < g.second; o += 16) {
        const int n = std::min(16, g.second - o);
        const int* wl = c->dwl + g.first + o;
        if (n <= 8) {
          const size_t sm = sizeof(float) * (2 * 32 * 8 + 2 * (size_t)gk);
          k_offdiag_D32g<8, 4><<<grid, 128, sm, s>>>(c->d_wires, wl, n, c->occf, c->dconst,
                                                      c->dpre, c->De, c->Dh);
        } else {
          const size_t sm = sizeof(float) * (2 * 32 * 16 + 2 * (size_t)gk);
          k_offdiag_D32g<16, 4><<<grid, 128, sm, s>>>(c->d_wires, wl, n, c->occf, c->dconst,
                                                       c->dpre, c->De, c->Dh);
        }
      }
    }
    return;
  }
  dim3 g((c->nk_max + 127) / 128, 2 * (2 * c->nk_max + 1), w_only >= 0 ? 1 : c->nw);
  double g0 = 0, g1 = 0, g2 = 0;
  int use_g = 0;
  if (g3) { g0 = g3[0]; g1 = g3[1]; g2 = g3[2]; use_g = 1; }
  k_offdiag_D64<<<g, 128, 0, s>>>(c->d_wires, w_only, c->ne, c->nh, c->Ee, c->Eh, c->vs, g0, g1,
                                  g2, use_g, c->De, c->Dh);
}

// dephasing.py:320-356: x = i hbar (A p + p B^T) with A[kh,j] = Dh[j-kh+Nk][kh],
// B[ke,j] = De[j-ke+Nk][ke] and the j = row entry removed (undel[q=0] = 0).
__global__ void k_offdiag_AB(const WireDev* wires, int w_only, const double* De,
                             const double* Dh, double2* A, double2* B) {
  int wi = (w_only >= 0) ? w_only : blockIdx.z;
  const WireDev W = wires[wi];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int row = blockIdx.y;
  if (row >= W.nk || j >= W.nk) return;
  int nk = W.nk;
  long long o = W.off_mat + (long long)row * nk + j;
  bool on = (w_only >= 0 || (W.flags & SBE_F_OFFDIAGDPH)) && j != row;
  long long di = W.off_dd + (long long)(j - row + nk) * nk + row;
  A[o] = make_double2(on ? Dh[di] : 0.0, 0.0);
  B[o] = make_double2(on ? De[di] : 0.0, 0.0);
}

void launch_offdiag_AB(SbeCtx* c, int w_only, cudaStream_t s) {
  dim3 g((c->nk_max + 127) / 128, c->nk_max, w_only >= 0 ? 1 : c->nw);
  k_offdiag_AB<<<g, 128, 0, s>>>(c->d_wires, w_only, c->De, c->Dh, c->dA, c->dB);
}

// ---------------------------------------------------------------------------
// Diagonal traces tr_d(X) = sum_k X[k][k+d], d in (-Nk, Nk), for the direct
// Coulomb terms of CalcH (SBEs.py:1094-1103).  Layout per wire: [2][2Nk] with
// entry d + Nk (C first, then D).
__global__ void k_traces(const WireDev* wires, const double2* C, const double2* D, double2* tr) {
  const WireDev W = wires[blockIdx.z];
  int nk = W.nk;
  int d = blockIdx.x - (nk - 1) + 0;  // blockIdx.x in [0, 2nk-1)
  int which = blockIdx.y;
  if ((int)blockIdx.x >= 2 * nk - 1) return;
  const double2* X = (which == 0 ? C : D) + W.off_mat;
  int k0 = d >= 0 ? 0 : -d, k1 = d >= 0 ? nk - 1 - d : nk - 1;
  double sr = 0.0, si = 0.0;
  for (int k = k0 + threadIdx.x; k <= k1; k += 32) {
    double2 v = X[(long long)k * nk + k + d];
    sr += v.x;
    si += v.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (threadIdx.x == 0) tr[4 * W.off_vec + which * 2 * nk + d + nk] = make_double2(sr, si);
}

void launch_traces(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s) {
  k_traces<<<dim3(2 * c->nk_max - 1, 2, c->nw), 32, 0, s>>>(c->d_wires, C, D, c->tr);
}

// ---------------------------------------------------------------------------
// SBEs.py:1044-1131 _CalcH_fallback and SBEs.py:5153-5163 _calc_Meh.
// V[n][q] = VC[|q|][0][n] for 1 <= |q| < Nk (given by vq, stride nk per n).
struct CalcHArgs {
  int nk, nr;
  const double2 *Meh, *Wee, *Whh, *C, *D, *P, *Ek;
  const double *vq, *Ee, *Eh;
  const double2* tr;    // [2][2nk] traces (C, D), may be null when !lf
  double gap, ehint, dcv;
  int yw, zsign, excitons, lf, freepot, optics;
  double2 *Heh, *Hee, *Hhh;
};

__device__ void calch_point(const CalcHArgs& a, int k1, int k2) {
  const int nk = a.nk;
  // Meh[ke=k1][kh=k2]
  double2 heh;
  if (a.Meh) {
    heh = a.Meh[(long long)k1 * nk + k2];
  } else if (a.Ek && a.optics) {
    int q = k1 - k2;
    if (q < 0) q += a.nr;
    double2 ex = a.Ek[q], ey = a.Ek[a.nr + q], ez = a.Ek[2 * a.nr + q];
    double xcv = a.dcv * ((k2 & 1) ? -1.0 : 1.0);
    double2 t1 = cscale(ex, -a.ehint * xcv);
    double2 t2 = cscale(cscale(ey, a.ehint * a.dcv), (double)a.yw);
    double2 t3 = cscale(cscale(ez, a.ehint * -a.dcv), (double)a.zsign);
    heh = csub(csub(t1, t2), t3);
  } else {
    heh = make_double2(0.0, 0.0);
  }
  double2 hee = make_double2(k1 == k2 ? a.Ee[k1] + a.gap : 0.0, 0.0);
  double2 hhh = make_double2(k1 == k2 ? a.Eh[k1] : 0.0, 0.0);
  if (a.freepot) {
    hee = cadd(hee, a.Wee[(long long)k1 * nk + k2]);
    hhh = cadd(hhh, a.Whh[(long long)k1 * nk + k2]);
  }
  if (a.excitons) {
    int qmin = max(-k1, -k2), qmax = min(nk - 1 - k1, nk - 1 - k2);
    const double* v0 = a.vq;
    const double* v1 = a.vq + nk;
    const double* v2 = a.vq + 2 * nk;
    for (int q = qmin; q <= qmax; ++q) {
      if (q == 0) continue;
      int aq = q < 0 ? -q : q;
      long long idx = (long long)(k2 + q) * nk + (k1 + q);   // X^T[k1+q][k2+q]
      double2 pv = a.P[idx];
      heh.x += v0[aq] * pv.x;
      heh.y += v0[aq] * pv.y;
    }
    if (a.lf) {
      for (int q = qmin; q <= qmax; ++q) {
        if (q == 0) continue;
        int aq = q < 0 ? -q : q;
        long long idx = (long long)(k2 + q) * nk + (k1 + q);
        double2 cv = a.C[idx], dv = a.D[idx];
        hee.x -= v1[aq] * cv.x;
        hee.y -= v1[aq] * cv.y;
        hhh.x -= v2[aq] * dv.x;
        hhh.y -= v2[aq] * dv.y;
      }
      int d = k1 - k2;
      if (d != 0) {
        int ad = d < 0 ? -d : d;
        double2 trC = a.tr[d + nk], trCm = a.tr[-d + nk];
        double2 trD = a.tr[2 * nk + d + nk], trDm = a.tr[2 * nk - d + nk];
        hee.x += v1[ad] * trC.x - v0[ad] * trDm.x;
        hee.y += v1[ad] * trC.y - v0[ad] * trDm.y;
        hhh.x += v2[ad] * trD.x - v0[ad] * trCm.x;
        hhh.y += v2[ad] * trD.y - v0[ad] * trCm.y;
      }
    } else if (k1 == k2) {
      for (int j = 0; j < nk; ++j) {
        if (j == k1) continue;
        int aq = j - k1 < 0 ? k1 - j : j - k1;
        double2 cv = a.C[(long long)j * nk + j], dv = a.D[(long long)j * nk + j];
        hee.x -= v1[aq] * cv.x;
        hee.y -= v1[aq] * cv.y;
        hhh.x -= v2[aq] * dv.x;
        hhh.y -= v2[aq] * dv.y;
      }
    }
  }
  long long o = (long long)k1 * nk + k2;
  a.Heh[o] = heh;
  a.Hee[o] = hee;
  a.Hhh[o] = hhh;
}

__global__ void k_calch_ctx(const WireDev* wires, const double2* P, const double2* C,
                            const double2* D, const double2* Ek, const double* vs,
                            const double* Ee, const double* Eh, const double2* tr, double2* Heh,
                            double2* Hee, double2* Hhh) {
  const WireDev W = wires[blockIdx.z];
  int k1 = blockIdx.x * blockDim.x + threadIdx.x;
  int k2 = blockIdx.y;
  if (k1 >= W.nk || k2 >= W.nk) return;
  CalcHArgs a;
  a.nk = W.nk;
  a.nr = W.nr;
  a.Meh = nullptr;
  a.Wee = a.Whh = nullptr;
  a.P = P + W.off_mat;
  a.C = C + W.off_mat;
  a.D = D + W.off_mat;
  a.Ek = Ek ? Ek + 3 * W.off_r : nullptr;
  a.vq = vs + 3 * W.off_vec;
  a.Ee = Ee + W.off_vec;
  a.Eh = Eh + W.off_vec;
  a.tr = tr + 4 * W.off_vec;
  a.gap = W.gap;
  a.ehint = W.ehint;
  a.dcv = W.dcv;
  a.yw = W.yw;
  a.zsign = W.zsign;
  a.excitons = (W.flags & SBE_F_EXCITONS) != 0;
  a.lf = (W.flags & SBE_F_LF) != 0;
  a.freepot = 0;
  a.optics = (W.flags & SBE_F_OPTICS) != 0;
  a.Heh = Heh + W.off_mat;
  a.Hee = Hee + W.off_mat;
  a.Hhh = Hhh + W.off_mat;
  calch_point(a, k1, k2);
}

void launch_calch_ctx(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                      const double2* Ek, cudaStream_t s) {
  launch_traces(c, C, D, s);
  dim3 g((c->nk_max + 63) / 64, c->nk_max, c->nw);
  k_calch_ctx<<<g, 64, 0, s>>>(c->d_wires, P, C, D, Ek, c->vs, c->Ee, c->Eh, c->tr, c->Heh,
                               c->Hee, c->Hhh);
}

// Single-wire CalcH on explicit arrays (the reference's pure-function call).
__global__ void k_vq_from_vc(int nk, const double* VC, double* vq) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nk) return;
  for (int n = 0; n < 3; ++n) vq[n * nk + q] = VC[((long long)q * nk + 0) * 3 + n];
}

__global__ void k_traces_single(int nk, const double2* C, const double2* D, double2* tr) {
  int d = (int)blockIdx.x - (nk - 1);
  int which = blockIdx.y;
  const double2* X = which == 0 ? C : D;
  int k0 = d >= 0 ? 0 : -d, k1 = d >= 0 ? nk - 1 - d : nk - 1;
  double sr = 0.0, si = 0.0;
  for (int k = k0 + threadIdx.x; k <= k1; k += 32) {
    double2 v = X[(long long)k * nk + k + d];
    sr += v.x;
    si += v.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (threadIdx.x == 0) tr[which * 2 * nk + d + nk] = make_double2(sr, si);
}

__global__ void k_calch_single(CalcHArgs a) {
  int k1 = blockIdx.x * blockDim.x + threadIdx.x;
  int k2 = blockIdx.y;
  if (k1 >= a.nk || k2 >= a.nk) return;
  calch_point(a, k1, k2);
}

int launch_calch_single(int nk, const double2* Meh, const double2* Wee, const double2* Whh,
                        const double2* C, const double2* D, const double2* P, const double* VC,
                        const double* Ee, const double* Eh, double gap, int excitons, int lf,
                        int freepot, double2* Heh, double2* Hee, double2* Hhh, cudaStream_t s) {
  double* vq = nullptr;
  double2* tr = nullptr;
  if (cudaMallocAsync(&vq, sizeof(double) * 3 * nk, s) != cudaSuccess ||
      cudaMallocAsync(&tr, sizeof(double2) * 4 * nk, s) != cudaSuccess)
    return fail(SBE_ERR_OOM, "sbe_calch: scratch allocation failed");
  k_vq_from_vc<<<(nk + 127) / 128, 128, 0, s>>>(nk, VC, vq);
  k_traces_single<<<dim3(2 * nk - 1, 2), 32, 0, s>>>(nk, C, D, tr);
  CalcHArgs a;
  a.nk = nk;
  a.nr = 2 * nk + 2;
  a.Meh = Meh;
  a.Wee = Wee;
  a.Whh = Whh;
  a.C = C;
  a.D = D;
  a.P = P;
  a.Ek = nullptr;
  a.vq = vq;
  a.Ee = Ee;
  a.Eh = Eh;
  a.tr = tr;
  a.gap = gap;
  a.ehint = a.dcv = 0.0;
  a.yw = a.zsign = 1;
  a.excitons = excitons;
  a.lf = lf;
  a.freepot = freepot;
  a.optics = 0;
  a.Heh = Heh;
  a.Hee = Hee;
  a.Hhh = Hhh;
  k_calch_single<<<dim3((nk + 63) / 64, nk), 64, 0, s>>>(a);
  cudaFreeAsync(vq, s);
  cudaFreeAsync(tr, s);
  return cuda_check(cudaGetLastError(), "sbe_calch");
}

}  // namespace sbe
