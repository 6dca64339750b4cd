// Mixed-precision (tcgen05) path of the SBE right-hand side: FP16 hi/lo plane
// conversion, per-wire power-of-two scaling and the self-test entry point.
#include <cuda_fp16.h>

#include "sbe_ctx.cuh"
#include "tc_gemm.cuh"

namespace sbe {

// ---------------------------------------------------------------------------
// max(|re|, |im|) of each batch entry of a packed complex array (float bits,
// atomicMax on the unsigned pattern of a non-negative float).
__global__ void k_absmax(const double2* X, long long per_batch, long long bstride, unsigned* out) {
  const int b = blockIdx.y;
  const double2* x = X + (long long)b * bstride;
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per_batch;
       i += (long long)gridDim.x * blockDim.x) {
    double2 v = x[i];
    m = fmaxf(m, (float)fmax(fabs(v.x), fabs(v.y)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out + b, __float_as_uint(m));
}

// e[b] = 14 - ceil(log2(max)): scaled magnitudes stay <= 2^14 (FP16 max 65504).
__global__ void k_exponents(int nb, const unsigned* mx, int* e, const int* add, int* sum) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  float m = __uint_as_float(mx[b]) * 1.0001f;
  int v = (m > 0.f) ? 14 - (int)ceilf(log2f(m)) : 0;
  e[b] = v;
  if (sum) sum[b] = v + (add ? add[b] : 0);
}

// FP16 hi/lo planes of a batch of Nk x Nk complex matrices, scaled by 2^e[b];
// optionally transposed.  dst layout [mat][plane][batch][rows][K]; planes
// re_hi, re_lo, im_hi, im_lo (complex) or hi, lo of the real part.
__global__ void k_planes(const double2* X, long long bstride, int nk, int transpose,
                         const int* e, __half* dst, int mat, int nplanes, int nbatch,
                         int real_only) {
  __shared__ double2 tile[32][33];
  const int b = blockIdx.z;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const double2* x = X + (long long)b * bstride;
  // output block: rows r0.., columns c0.. of Y (Y = X or X^T).  For X^T the
  // tile holds X[c0 + i][r0 + j]; reads and writes are coalesced along x.
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int r = (transpose ? c0 : r0) + i, c = (transpose ? r0 : c0) + threadIdx.x;
    tile[i][threadIdx.x] = (r < nk && c < nk) ? x[(long long)r * nk + c] : make_double2(0, 0);
  }
  __syncthreads();
  const double sc = ldexp(1.0, e[b]);
  const long long plane = (long long)nbatch * nk * nk;
  __half* base = dst + ((long long)mat * nplanes) * plane + (long long)b * nk * nk;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int r = r0 + i, c = c0 + threadIdx.x;
    if (r >= nk || c >= nk) continue;
    double2 v = transpose ? tile[threadIdx.x][i] : tile[i][threadIdx.x];
    long long o = (long long)r * nk + c;
    // scale in FP64 (exact), round once to FP32 (24 bits >= the 22 the planes
    // keep) and split in FP32: the FP64 pipe is the scarce one on GB300
    const float vr = (float)(v.x * sc), vi = (float)(v.y * sc);
    const __half rh = __float2half_rn(vr);
    base[o] = rh;
    base[plane + o] = __float2half_rn(vr - __half2float(rh));
    if (!real_only) {
      const __half ih = __float2half_rn(vi);
      base[2 * plane + o] = ih;
      base[3 * plane + o] = __float2half_rn(vi - __half2float(ih));
    }
  }
}

void launch_planes(const double2* X, long long bstride, int nk, int nbatch, int transpose,
                   const int* e, __half* dst, int mat, int nplanes, int real_only,
                   cudaStream_t s) {
  dim3 blk(32, 8), grid((nk + 31) / 32, (nk + 31) / 32, nbatch);
  k_planes<<<grid, blk, 0, s>>>(X, bstride, nk, transpose, e, dst, mat, nplanes, nbatch,
                                real_only);
}

void launch_exponents(const double2* X, long long per_batch, long long bstride, int nbatch,
                      unsigned* mx, int* e, const int* add, int* sum, cudaStream_t s) {
  cudaMemsetAsync(mx, 0, sizeof(unsigned) * nbatch, s);
  int blocks = (int)std::min<long long>((per_batch + 255) / 256, 256);
  k_absmax<<<dim3(blocks, nbatch), 256, 0, s>>>(X, per_batch, bstride, mx);
  k_exponents<<<(nbatch + 127) / 128, 128, 0, s>>>(nbatch, mx, e, add, sum);
}

// ---------------------------------------------------------------------------
// Mixed-precision workspace of a context (uniform Nk and flags over its wires).
//
// Commutator planes: 14 matrices x 4 planes x Nw x Nk x Nk (FP16):
//   0 P, 1 P^T, 2 C, 3 C^T, 4 D, 5 D^T            (state, exponent eS)
//   6 Heh, 7 Heh^T, 8 Hee', 9 Hee'^T, 10 Hhh', 11 Hhh'^T,
//   12 Hee' + i hbar B, 13 Hhh' + i hbar A         (Hamiltonians, exponent eH)
// (' = diagonal removed; A, B = off-diagonal dephasing matrices).
// Exchange: Toeplitz planes T_n (3 x 2 x Nw x Nk x Nk) and sheared state planes
// S_n (3 x 2 x Nw x 4Nk x Nk).  Sources: E^T planes (4 x Nw x Nr x Nk).
struct Mixed {
  int nk = 0, nw = 0, nr = 0;
  __half *planes = nullptr, *tpl = nullptr, *spl = nullptr, *epl = nullptr;
  float* xsh = nullptr;  // exchange sums in the sheared layout: 3 x Nw x Nk x 4Nk
  int* ints = nullptr;   // eS, eH, eT, eE, esc, esx, ess, err  (8 x nw)
  unsigned* mx = nullptr;
  double2 *dgE = nullptr, *dgH = nullptr;
  CUtensorMap mapA, mapB, mapTA, mapSB, mapEB;
  int* eS() { return ints; }
  int* eH() { return ints + nw; }
  int* eT() { return ints + 2 * nw; }
  int* eE() { return ints + 3 * nw; }
  int* esc() { return ints + 4 * nw; }
  int* esx() { return ints + 5 * nw; }
  int* ess() { return ints + 6 * nw; }
  int* err() { return ints + 7 * nw; }
};

enum { M_P = 0, M_PT, M_C, M_CT, M_D, M_DT, M_EH, M_EHT, M_EE, M_EET, M_HH, M_HHT, M_EEX, M_HHX };

void mixed_free(SbeCtx* c) {
  Mixed* m = static_cast<Mixed*>(c->mixed);
  if (!m) return;
  cudaFree(m->planes);
  cudaFree(m->tpl);
  cudaFree(m->spl);
  cudaFree(m->epl);
  cudaFree(m->xsh);
  cudaFree(m->ints);
  cudaFree(m->mx);
  cudaFree(m->dgE);
  delete m;
  c->mixed = nullptr;
}

// E^T planes: Y[r][k] = Expikr[k][r] (|E| = 1, exponent 13).
__global__ void k_eplanes(const WireDev* wires, const double2* expikr, __half* dst, int nw) {
  const WireDev W = wires[blockIdx.z];
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  int r = blockIdx.y;
  if (k >= W.nk || r >= W.nr) return;
  double2 v = expikr[W.off_kr + (long long)k * W.nr + r];
  const long long plane = (long long)nw * W.nr * W.nk;
  long long o = (long long)blockIdx.z * W.nr * W.nk + (long long)r * W.nk + k;
  double vr = ldexp(v.x, 13), vi = ldexp(v.y, 13);
  __half rh = __double2half(vr), ih = __double2half(vi);
  dst[o] = rh;
  dst[plane + o] = __double2half(vr - (double)__half2float(rh));
  dst[2 * plane + o] = ih;
  dst[3 * plane + o] = __double2half(vi - (double)__half2float(ih));
}

__global__ void k_fill_int(int* p, int n, int v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

static int mixed_ensure(SbeCtx* c, cudaStream_t s) {
  if (c->mixed) return SBE_OK;
  const int nk = c->wires[0].nk, nw = c->nw;
  for (int w = 1; w < nw; ++w)
    if (c->wires[w].nk != nk || c->wires[w].flags != c->wires[0].flags)
      return fail(SBE_ERR_UNSUPPORTED,
                  "mixed path: all wires of a context must share Nk and flags (group by Nk)");
  if (nk % 8) return fail(SBE_ERR_UNSUPPORTED, "mixed path: Nk must be a multiple of 8");
  Mixed* m = new Mixed();
  m->nk = nk;
  m->nw = nw;
  m->nr = 2 * nk + 2;
  const size_t mm = (size_t)nk * nk;
  bool ok = cudaMalloc(&m->planes, sizeof(__half) * 14 * 4 * nw * mm) == cudaSuccess &&
            cudaMalloc(&m->tpl, sizeof(__half) * 3 * 2 * nw * mm) == cudaSuccess &&
            cudaMalloc(&m->spl, sizeof(__half) * 3 * 2 * nw * 4 * mm) == cudaSuccess &&
            cudaMalloc(&m->epl, sizeof(__half) * 4 * nw * (size_t)m->nr * nk) == cudaSuccess &&
            cudaMalloc(&m->xsh, sizeof(float) * 3 * nw * 4 * mm) == cudaSuccess &&
            cudaMalloc(&m->ints, sizeof(int) * 8 * nw) == cudaSuccess &&
            cudaMalloc(&m->mx, sizeof(unsigned) * nw) == cudaSuccess &&
            cudaMalloc(&m->dgE, sizeof(double2) * 2 * nw * nk) == cudaSuccess;
  if (!ok) {
    c->mixed = m;
    mixed_free(c);
    return fail(SBE_ERR_OOM, "mixed path: workspace allocation failed");
  }
  m->dgH = m->dgE + (size_t)nw * nk;
  cudaMemsetAsync(m->ints, 0, sizeof(int) * 8 * nw, s);
  TcPlanes pl{m->planes, 14, 4, nw, nk, nk};
  TcPlanes tp{m->tpl, 3, 2, nw, nk, nk};
  TcPlanes sp{m->spl, 3, 2, nw, 4 * nk, nk};
  TcPlanes ep{m->epl, 1, 4, nw, m->nr, nk};
  int rc = tc_make_maps(pl, pl, &m->mapA, &m->mapB);
  if (!rc) rc = tc_make_maps(tp, sp, &m->mapTA, &m->mapSB);
  CUtensorMap dummy;
  if (!rc) rc = tc_make_maps(tp, ep, &dummy, &m->mapEB);
  if (rc) {
    c->mixed = m;
    mixed_free(c);
    return rc;
  }
  k_eplanes<<<dim3((nk + 127) / 128, m->nr, nw), 128, 0, s>>>(c->d_wires, c->expikr, m->epl, nw);
  k_fill_int<<<(nw + 127) / 128, 128, 0, s>>>(m->eE(), nw, 13);
  c->mixed = m;
  return cuda_check(cudaGetLastError(), "mixed workspace");
}

// generic per-batch max over several arrays (scaled by fac)
__global__ void k_absmax_f(const double2* X, long long per_batch, long long bstride, double fac,
                           unsigned* out) {
  const int b = blockIdx.y;
  const double2* x = X + (long long)b * bstride;
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per_batch;
       i += (long long)gridDim.x * blockDim.x) {
    double2 v = x[i];
    m = fmaxf(m, (float)(fac * fmax(fabs(v.x), fabs(v.y))));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out + b, __float_as_uint(m));
}

static void absmax_into(const double2* X, long long per, int nw, double fac, unsigned* mx,
                        cudaStream_t s) {
  int blocks = (int)std::min<long long>((per + 255) / 256, 128);
  k_absmax_f<<<dim3(blocks, nw), 256, 0, s>>>(X, per, per, fac, mx);
}

// Toeplitz exchange planes T_n[t][t'] = vs_n(|t - t'|) (t != t'), real.
__global__ void k_toeplitz_planes(const WireDev* wires, const double* vs, const int* e,
                                  __half* dst, int nw) {
  const int b = blockIdx.z / 3, n = blockIdx.z % 3;
  const WireDev W = wires[b];
  const int nk = W.nk;
  int tp = blockIdx.x * blockDim.x + threadIdx.x;
  int t = blockIdx.y;
  if (tp >= nk || t >= nk) return;
  int d = t > tp ? t - tp : tp - t;
  double v = (d == 0) ? 0.0 : ldexp(vs[3 * W.off_vec + n * nk + d], e[b]);
  const long long mm = (long long)nk * nk, plane = (long long)nw * mm;
  __half* base = dst + (long long)n * 2 * plane + (long long)b * mm + (long long)t * nk + tp;
  __half h = __double2half(v);
  base[0] = h;
  base[plane] = __double2half(v - (double)__half2float(h));
}

__global__ void k_vs_max(const WireDev* wires, const double* vs, unsigned* mx) {
  const WireDev W = wires[blockIdx.x];
  float m = 0.f;
  for (int i = threadIdx.x; i < 3 * W.nk; i += blockDim.x)
    m = fmaxf(m, (float)fabs(vs[3 * W.off_vec + i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx + blockIdx.x, __float_as_uint(m));
}

// Sheared state planes: row 2 dd + c (dd = d + Nk - 1, c = re / im), column t':
// S[2dd + c][t'] = component c of X[t' + d][t'] (zero outside the matrix).
// The exchange sum  H[t][t+d] = sum_t' V(|t - t'|) X[t' + d][t']  is then T S.
__global__ void k_shear_planes(int nk, int nw, const double2* X, const int* e, __half* dst,
                               int mat) {
  const int b = blockIdx.z;
  const int tp = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = blockIdx.y;   // 0 .. 4nk-1
  if (tp >= nk) return;
  const int dd = row >> 1, c = row & 1;
  const int d = dd - (nk - 1);
  float v = 0.f;
  if (dd < 2 * nk - 1 && tp + d >= 0 && tp + d < nk) {
    const double* x = reinterpret_cast<const double*>(
        X + (long long)b * nk * nk + (long long)(tp + d) * nk + tp);
    v = (float)(x[c] * ldexp(1.0, e[b]));
  }
  const long long rows = 4ll * nk, plane = (long long)nw * rows * nk;
  __half* base = dst + (long long)mat * 2 * plane + (long long)b * rows * nk + (long long)row * nk + tp;
  const __half h = __float2half_rn(v);
  base[0] = h;
  base[plane] = __float2half_rn(v - __half2float(h));
}

// H = Meh + diagonal energies + direct Coulomb terms + exchange sums
// (SBEs.py:1044-1131).  The exchange sums come from the sheared FP32 GEMM output
// xsh[n][b][k1][2 dd + c], dd = k2 - k1 + Nk - 1, which is read along rows
// (coalesced in k2).  The diagonal of Hee / Hhh is split off into dgE / dgH
// (the GEMM operands carry H' = H - diag); the max |component| of the
// operands goes to mx[b].
__global__ void k_h_build(const WireDev* wires, const double2* Ek, const double* vs,
                          const double* Ee, const double* Eh, const double2* tr, const float* xsh,
                          int have_x, double2* Heh, double2* Hee, double2* Hhh, double2* dgE,
                          double2* dgH, unsigned* mx) {
  const WireDev& W = wires[blockIdx.z];
  const int nk = W.nk;
  const int k2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int k1 = blockIdx.y;
  float hmax = 0.f;
  if (k1 < nk && k2 < nk) {
    // off-diagonal elements in FP32 (they only feed the FP16 hi/lo operands and
    // the driving term of dP); the diagonal (gap + kinetic energy) in FP64
    float2 heh = make_float2(0.f, 0.f), hee = heh, hhh = heh;
    if (W.flags & SBE_F_OPTICS) {
      int q = k1 - k2;
      if (q < 0) q += W.nr;
      const double2* ek = Ek + 3 * W.off_r;
      double2 ex = ek[q], ey = ek[W.nr + q], ez = ek[2 * W.nr + q];
      const float ed = (float)(W.ehint * W.dcv);
      const float sx = (k2 & 1) ? ed : -ed;               // -ehint Xcv
      const float sy = -ed * (float)W.yw, sz = ed * (float)W.zsign;
      heh.x = sx * (float)ex.x + sy * (float)ey.x + sz * (float)ez.x;
      heh.y = sx * (float)ex.y + sy * (float)ey.y + sz * (float)ez.y;
    }
    const bool exc = (W.flags & SBE_F_EXCITONS) != 0, lf = (W.flags & SBE_F_LF) != 0;
    const int d = k1 - k2;
    if (exc && lf && d != 0) {
      const double* v = vs + 3 * W.off_vec;
      const double2* t = tr + 4 * W.off_vec;
      const int ad = d < 0 ? -d : d;
      const float v0 = (float)v[ad], v1 = (float)v[nk + ad], v2 = (float)v[2 * nk + ad];
      double2 trC = t[d + nk], trCm = t[-d + nk], trD = t[2 * nk + d + nk],
              trDm = t[2 * nk - d + nk];
      hee.x = v1 * (float)trC.x - v0 * (float)trDm.x;
      hee.y = v1 * (float)trC.y - v0 * (float)trDm.y;
      hhh.x = v2 * (float)trD.x - v0 * (float)trCm.x;
      hhh.y = v2 * (float)trD.y - v0 * (float)trCm.y;
    }
    float2 xc = make_float2(0.f, 0.f), xd = xc;
    if (have_x) {
      const long long ms = (long long)nk * 4 * nk;
      const long long rowo = ((long long)blockIdx.z * nk + k1) * 4 * nk + 2 * (k2 - k1 + nk - 1);
      const long long plane = (long long)gridDim.z * ms;
      float2 xe = *reinterpret_cast<const float2*>(xsh + rowo);
      heh.x += xe.x;
      heh.y += xe.y;
      if (lf || d == 0) {
        xc = *reinterpret_cast<const float2*>(xsh + plane + rowo);
        xd = *reinterpret_cast<const float2*>(xsh + 2 * plane + rowo);
      }
    }
    const long long o = W.off_mat + (long long)k1 * nk + k2;
    Heh[o] = make_double2(heh.x, heh.y);
    if (d == 0) {
      const long long vo = (long long)blockIdx.z * nk + k1;
      dgE[vo] = make_double2(Ee[W.off_vec + k1] + W.gap - (double)xc.x, -(double)xc.y);
      dgH[vo] = make_double2(Eh[W.off_vec + k1] - (double)xd.x, -(double)xd.y);
      hee = make_float2(0.f, 0.f);
      hhh = hee;
    } else {
      hee.x -= xc.x;
      hee.y -= xc.y;
      hhh.x -= xd.x;
      hhh.y -= xd.y;
    }
    Hee[o] = make_double2(hee.x, hee.y);
    Hhh[o] = make_double2(hhh.x, hhh.y);
    hmax = fmaxf(fmaxf(fmaxf(fabsf(heh.x), fabsf(heh.y)), fmaxf(fabsf(hee.x), fabsf(hee.y))),
                 fmaxf(fabsf(hhh.x), fabsf(hhh.y)));
  }
  for (int o = 16; o > 0; o >>= 1) hmax = fmaxf(hmax, __shfl_down_sync(0xffffffffu, hmax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx + blockIdx.z, __float_as_uint(hmax));
}

// planes with an added i * f * M (M real-valued complex array), used for
// Hee' + i hbar B and Hhh' + i hbar A.
__global__ void k_planes_add(const double2* X, const double2* Madd, double f, int nk,
                             const int* e, __half* dst, int mat, int nw) {
  const int b = blockIdx.z;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  int r = blockIdx.y;
  if (c >= nk || r >= nk) return;
  const long long mm = (long long)nk * nk, plane = (long long)nw * mm;
  long long o = (long long)r * nk + c;
  double2 v = X[(long long)b * mm + o];
  double2 a = Madd[(long long)b * mm + o];
  const double sc = ldexp(1.0, e[b]);
  const float vr = (float)((v.x - f * a.y) * sc), vi = (float)((v.y + f * a.x) * sc);
  __half* base = dst + (long long)mat * 4 * plane + (long long)b * mm + o;
  const __half rh = __float2half_rn(vr), ih = __float2half_rn(vi);
  base[0] = rh;
  base[plane] = __float2half_rn(vr - __half2float(rh));
  base[2 * plane] = ih;
  base[3 * plane] = __float2half_rn(vi - __half2float(ih));
}

// dC (dD) from W = C Hee'^T + P^H Heh^T (V = D Hhh'^T + conj(P) Heh): for
// Hermitian C, Hee (D, Hhh) the four terms of dCdt (dDdt) are W - W^H, so
//   dX[i][j] = (W[i][j] - conj(W[j][i]) + (g[j] - g[i]) X[i][j]) / (i hbar)
// with g the peeled diagonal.  The result is exactly anti-Hermitian, which
// keeps C and D Hermitian.  Tiles (bi, bj) and (bj, bi) meet in shared memory.
__global__ void k_antiherm(int nk, const double2* W, long long wb, const double2* X,
                           const double2* g, double2* out) {
  __shared__ double2 t[32][33];
  const int b = blockIdx.z;
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const double2* w = W + (long long)b * wb;
  const long long mb = (long long)b * nk * nk;
  // t[jj][ii] = W[j0 + jj][i0 + ii]   (the transposed tile)
  for (int jj = threadIdx.y; jj < 32; jj += blockDim.y) {
    int r = j0 + jj, cc = i0 + threadIdx.x;
    t[jj][threadIdx.x] = (r < nk && cc < nk) ? w[(long long)r * nk + cc] : make_double2(0, 0);
  }
  __syncthreads();
  const double ih = 1.0 / kHbar;
  for (int ii = threadIdx.y; ii < 32; ii += blockDim.y) {
    int i = i0 + ii, j = j0 + threadIdx.x;
    if (i >= nk || j >= nk) continue;
    double2 a = w[(long long)i * nk + j];
    double2 bT = t[threadIdx.x][ii];                 // W[j][i]
    double2 x = X[mb + (long long)i * nk + j];
    double2 gi = g[(long long)b * nk + i], gj = g[(long long)b * nk + j];
    double2 de = make_double2(gj.x - gi.x, gj.y - gi.y);
    double2 dx = make_double2(de.x * x.x - de.y * x.y, de.x * x.y + de.y * x.x);
    double re = a.x - bT.x + dx.x, im = a.y + bT.y + dx.y;
    out[mb + (long long)i * nk + j] = make_double2(im * ih, -re * ih);
  }
}

__global__ void k_add_int(int n, const int* a, const int* b, int* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}

static int gemm(Mixed* m, const CUtensorMap& A, const CUtensorMap& B, int M, int N, int K, int cplx,
                int nterms, const tc::Term* t, int kskip, const tc::EpiArgs& e, cudaStream_t s) {
  tc::GemmDesc d{};
  d.M = M;
  d.N = N;
  d.K = K;
  d.complex_mode = cplx;
  d.nterms = nterms;
  for (int i = 0; i < nterms; ++i) d.t[i] = t[i];
  d.batch = m->nw;
  d.kskip = kskip;
  d.nk_shear = m->nk;
  return tc_gemm_launch(d, A, B, e, s);
}

static void exponents_from_mx(Mixed* m, int* e, cudaStream_t s) {
  k_exponents<<<(m->nw + 127) / 128, 128, 0, s>>>(m->nw, m->mx, e, nullptr, nullptr);
}

// Per-step set-up of the mixed path: the frozen preparation (screening, rates,
// dephasing matrices with the FP32 Lorentzian sums) and the Toeplitz planes.
static int mixed_prep(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s) {
  Mixed* m = static_cast<Mixed*>(c->mixed);
  launch_prep_scalar(c, C, D, s);
  launch_gamma(c, -1, s);
  if (c->any_offdiag) {
    {
      ProfScope ps(c, 3, s);
      launch_offdiag_D(c, -1, nullptr, true, s);
    }
    launch_offdiag_AB(c, -1, s);
  } else {
    cudaMemsetAsync(c->dA, 0, sizeof(double2) * c->tot_mat, s);
    cudaMemsetAsync(c->dB, 0, sizeof(double2) * c->tot_mat, s);
  }
  cudaMemsetAsync(m->mx, 0, sizeof(unsigned) * m->nw, s);
  k_vs_max<<<m->nw, 256, 0, s>>>(c->d_wires, c->vs, m->mx);
  exponents_from_mx(m, m->eT(), s);
  k_toeplitz_planes<<<dim3((m->nk + 127) / 128, m->nk, 3 * m->nw), 128, 0, s>>>(
      c->d_wires, c->vs, m->eT(), m->tpl, m->nw);
  return cuda_check(cudaGetLastError(), "mixed prep");
}

// One stage RHS of every wire at state (P, C, D) and wire-k field Ek.
static int mixed_stage(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                       const double2* Ek, double2* dP, double2* dC, double2* dD,
                       cudaStream_t s) {
  Mixed* m = static_cast<Mixed*>(c->mixed);
  const int nk = m->nk, nw = m->nw;
  const long long mm = (long long)nk * nk;
  const WireDev& W0 = c->wires[0];
  // state exponent and planes
  cudaMemsetAsync(m->mx, 0, sizeof(unsigned) * nw, s);
  absmax_into(P, mm, nw, 1.0, m->mx, s);
  absmax_into(C, mm, nw, 1.0, m->mx, s);
  absmax_into(D, mm, nw, 1.0, m->mx, s);
  exponents_from_mx(m, m->eS(), s);
  const double2* st[3] = {P, C, D};
  for (int i = 0; i < 3; ++i) {
    launch_planes(st[i], mm, nk, nw, 0, m->eS(), m->planes, 2 * i, 4, 0, s);
    launch_planes(st[i], mm, nk, nw, 1, m->eS(), m->planes, 2 * i + 1, 4, 0, s);
  }
  // exchange sums (sheared GEMMs, FP32 output), then the Hamiltonians: Meh +
  // diagonal + direct + exchange, diagonal peeled, maximum for the H exponent
  launch_traces(c, C, D, s);
  int rc = SBE_OK;
  const int have_x = (W0.flags & SBE_F_EXCITONS) ? 1 : 0;
  if (have_x) {
    k_add_int<<<(nw + 127) / 128, 128, 0, s>>>(nw, m->eT(), m->eS(), m->esx());
    for (int n = 0; n < 3; ++n) {
      k_shear_planes<<<dim3((nk + 127) / 128, 4 * nk, nw), 128, 0, s>>>(nk, nw, st[n], m->eS(),
                                                                        m->spl, n);
      tc::Term t{n, n, 0, 0, 1};
      tc::EpiArgs e{};
      e.kind = tc::EPI_F32;
      e.outf = m->xsh + (long long)n * nw * 4 * mm;
      e.out_bstride = 4 * mm;
      e.escale = m->esx();
      e.err = m->err();
      ProfScope ps(c, 1, s);
      rc = gemm(m, m->mapTA, m->mapSB, nk, 4 * nk, nk, 0, 1, &t, 1, e, s);
      if (rc) return rc;
    }
  }
  cudaMemsetAsync(m->mx, 0, sizeof(unsigned) * nw, s);
  k_h_build<<<dim3((nk + 127) / 128, nk, nw), 128, 0, s>>>(c->d_wires, Ek, c->vs, c->Ee, c->Eh,
                                                           c->tr, m->xsh, have_x, c->Heh, c->Hee,
                                                           c->Hhh, m->dgE, m->dgH, m->mx);
  if (c->any_offdiag) {
    absmax_into(c->dA, mm, nw, 2.0 * kHbar, m->mx, s);
    absmax_into(c->dB, mm, nw, 2.0 * kHbar, m->mx, s);
  }
  exponents_from_mx(m, m->eH(), s);
  const double2* hs[3] = {c->Heh, c->Hee, c->Hhh};
  for (int i = 0; i < 3; ++i) {
    launch_planes(hs[i], mm, nk, nw, 0, m->eH(), m->planes, M_EH + 2 * i, 4, 0, s);
    if (i == 0)   // Hee'^T and Hhh'^T are not needed in the W - W^H form
      launch_planes(hs[i], mm, nk, nw, 1, m->eH(), m->planes, M_EH + 2 * i + 1, 4, 0, s);
  }
  dim3 pg((nk + 127) / 128, nk, nw);
  k_planes_add<<<pg, 128, 0, s>>>(c->Hee, c->dB, kHbar, nk, m->eH(), m->planes, M_EEX, nw);
  k_planes_add<<<pg, 128, 0, s>>>(c->Hhh, c->dA, kHbar, nk, m->eH(), m->planes, M_HHX, nw);
  k_add_int<<<(nw + 127) / 128, 128, 0, s>>>(nw, m->eS(), m->eH(), m->esc());
  // commutator GEMMs (term lists follow dpdt, SBEs.py:1942-1965; dCdt and dDdt,
  // SBEs.py:2309-2327 and 2607-2625, through their W - W^H form)
  const tc::Term tP[4] = {{M_HHX, M_PT, 0, 0, 1}, {M_DT, M_EH, 0, 0, -1},
                          {M_P, M_EEX, 0, 0, 1}, {M_EHT, M_CT, 0, 0, -1}};
  const tc::Term tC[2] = {{M_C, M_EE, 0, 0, 1}, {M_PT, M_EH, 1, 0, 1}};
  const tc::Term tD[2] = {{M_D, M_HH, 0, 0, 1}, {M_P, M_EHT, 1, 0, 1}};
  const tc::Term* tl[3] = {tP, tC, tD};
  const int nt[3] = {4, 2, 2};
  double2* Wbuf[3] = {dP, c->G, c->G + c->tot_kr};
  for (int w = 0; w < 3; ++w) {
    tc::EpiArgs e{};
    e.kind = (w == 0) ? tc::EPI_RHS : tc::EPI_RAW;
    e.which = w;
    e.out = Wbuf[w];
    e.out_bstride = mm;
    e.escale = m->esc();
    e.X = st[w];
    e.Heh = c->Heh;
    e.dgE = m->dgE;
    e.dgH = m->dgH;
    e.gamE = c->gamE;
    e.gamH = c->gamH;
    e.nk = nk;
    e.err = m->err();
    ProfScope ps(c, 0, s);
    rc = gemm(m, m->mapA, m->mapB, nk, nk, nk, 1, nt[w], tl[w], 0, e, s);
    if (rc) return rc;
  }
  dim3 ag((nk + 31) / 32, (nk + 31) / 32, nw), ab(32, 8);
  k_antiherm<<<ag, ab, 0, s>>>(nk, c->G, mm, C, m->dgE, dC);
  k_antiherm<<<ag, ab, 0, s>>>(nk, c->G + c->tot_kr, mm, D, m->dgH, dD);
  return cuda_check(cudaGetLastError(), "mixed stage");
}

// Sources of the new state through the engine: G = [P; C; conj(D)] E.
static int mixed_sources(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                         double2* src, cudaStream_t s) {
  Mixed* m = static_cast<Mixed*>(c->mixed);
  const int nk = m->nk, nw = m->nw;
  const long long mm = (long long)nk * nk;
  cudaMemsetAsync(m->mx, 0, sizeof(unsigned) * nw, s);
  absmax_into(P, mm, nw, 1.0, m->mx, s);
  absmax_into(C, mm, nw, 1.0, m->mx, s);
  absmax_into(D, mm, nw, 1.0, m->mx, s);
  exponents_from_mx(m, m->eS(), s);
  const double2* st[3] = {P, C, D};
  for (int i = 0; i < 3; ++i) launch_planes(st[i], mm, nk, nw, 0, m->eS(), m->planes, 2 * i, 4, 0, s);
  k_add_int<<<(nw + 127) / 128, 128, 0, s>>>(nw, m->eS(), m->eE(), m->ess());
  for (int i = 0; i < 3; ++i) {
    tc::Term t{2 * i, 0, i == 2 ? 1 : 0, 0, 1};
    tc::EpiArgs e{};
    e.kind = tc::EPI_RAW;
    e.out = c->G + i * c->tot_kr;
    e.out_bstride = (long long)nk * m->nr;
    e.escale = m->ess();
    e.err = m->err();
    ProfScope ps(c, 2, s);
    int rc = gemm(m, m->mapA, m->mapEB, nk, m->nr, nk, 1, 1, &t, 0, e, s);
    if (rc) return rc;
  }
  launch_sources_reduce(c, c->ne, c->nh, src, s);
  return cuda_check(cudaGetLastError(), "mixed sources");
}

int mixed_prepare(SbeCtx* c, cudaStream_t s) {
  int rc = mixed_ensure(c, s);
  if (rc) return rc;
  return tc_gemm_init();
}

int rhs_mixed(SbeCtx* c, const double2* P, const double2* C, const double2* D, const double2* Ek,
              double2* dP, double2* dC, double2* dD, cudaStream_t s) {
  // sbe_rhs has run the FP64 preparation; the mixed call redoes it with the
  // FP32 dephasing sums so that it measures exactly what the RK4 stages use.
  int rc = mixed_ensure(c, s);
  if (rc) return rc;
  rc = mixed_prep(c, C, D, s);
  if (rc) return rc;
  return mixed_stage(c, P, C, D, Ek, dP, dC, dD, s);
}

int rk4_mixed(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek0,
              const double2* dEk, double dt, double2* src, cudaStream_t s) {
  int rc = mixed_ensure(c, s);
  if (rc) return rc;
  rc = mixed_prep(c, C, D, s);
  if (rc) return rc;
  const long long n = c->tot_mat;
  const double frac[4] = {0.0, 0.5, 0.5, 1.0};
  for (int st = 1; st <= 4; ++st) {
    const double2 *xp = P, *xc = C, *xd = D;
    if (st > 1) {
      xp = c->xs;
      xc = c->xs + n;
      xd = c->xs + 2 * n;
    }
    launch_stage_field(c, Ek0, dEk, frac[st - 1], s);
    rc = mixed_stage(c, xp, xc, xd, c->ekst, c->dP, c->dC, c->dD, s);
    if (rc) return rc;
    launch_rk4_axpy(c, st, dt, P, C, D, s);
  }
  launch_relax_norm(c, C, D, dt, false, s);
  return mixed_sources(c, P, C, D, src, s);
}

}  // namespace sbe

using namespace sbe;

extern "C" int sbe_tc_selftest(int nk, int nbatch, const double* A, const double* B, int opA,
                               int opB, int complex_mode, double* out, void* stream) {
  if (nk < 8 || nk % 8 || nbatch < 1 || !A || !B || !out || opA < 0 || opA > 3 || opB < 0 ||
      opB > 3)
    return fail(SBE_ERR_ARG, "sbe_tc_selftest: bad arguments (nk must be a multiple of 8)");
  cudaStream_t s = as_stream(stream);
  const int npl = complex_mode ? 4 : 2;
  const long long mm = (long long)nk * nk;
  __half* planes = nullptr;
  int* ints = nullptr;
  unsigned* mx = nullptr;
  size_t pbytes = sizeof(__half) * 2 * npl * nbatch * mm;
  if (cudaMallocAsync(&planes, pbytes, s) != cudaSuccess ||
      cudaMallocAsync(&ints, sizeof(int) * (3 * nbatch + 1), s) != cudaSuccess ||
      cudaMallocAsync(&mx, sizeof(unsigned) * nbatch, s) != cudaSuccess)
    return fail(SBE_ERR_OOM, "sbe_tc_selftest: scratch");
  int* eA = ints;
  int* eB = ints + nbatch;
  int* es = ints + 2 * nbatch;
  int* err = ints + 3 * nbatch;
  cudaMemsetAsync(err, 0, sizeof(int), s);
  const double2* a2 = (const double2*)A;
  const double2* b2 = (const double2*)B;
  launch_exponents(a2, mm, mm, nbatch, mx, eA, nullptr, nullptr, s);
  launch_exponents(b2, mm, mm, nbatch, mx, eB, eA, es, s);
  // op(A)[m][k]: transposed for T/H; op(B)[k][n] as B-operand rows n: Y[n][k]
  const int tA = (opA == 1 || opA == 3), cA = (opA == 2 || opA == 3);
  const int tB = !(opB == 1 || opB == 3), cB = (opB == 2 || opB == 3);
  launch_planes(a2, mm, nk, nbatch, tA, eA, planes, 0, npl, !complex_mode, s);
  launch_planes(b2, mm, nk, nbatch, tB, eB, planes, 1, npl, !complex_mode, s);
  TcPlanes pl;
  pl.ptr = planes;
  pl.nmat = 2;
  pl.nplanes = npl;
  pl.batch = nbatch;
  pl.rows = nk;
  pl.K = nk;
  CUtensorMap ma, mb;
  int rc = tc_make_maps(pl, pl, &ma, &mb);
  if (rc) return rc;
  tc::GemmDesc d{};
  d.M = d.N = d.K = nk;
  d.complex_mode = complex_mode ? 1 : 0;
  d.nterms = 1;
  d.t[0] = tc::Term{0, 1, cA, cB, 1};
  d.batch = nbatch;
  tc::EpiArgs e{};
  e.kind = tc::EPI_RAW;
  e.out = (double2*)out;
  e.out_bstride = mm;
  e.escale = es;
  e.err = err;
  rc = tc_gemm_launch(d, ma, mb, e, s);
  if (rc) return rc;
  int herr = 0;
  cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  rc = cuda_check(cudaStreamSynchronize(s), "sbe_tc_selftest");
  cudaFreeAsync(planes, s);
  cudaFreeAsync(ints, s);
  cudaFreeAsync(mx, s);
  if (rc) return rc;
  if (herr) return fail(SBE_ERR_TIMEOUT, "sbe_tc_selftest: a pipeline wait timed out");
  return SBE_OK;
}
