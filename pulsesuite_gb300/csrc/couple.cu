// Coupling of a batch of wires to the 1-D PSTD grid, and the coupled time step.
//
// Field -> wire: Prop2QW (PSTD3D/qwoptics.py:667-715) with the grid seen from the
// wire: the Forsythe-Malcolm-Moler spline of each grid field (spliner.py:1329-1394),
// evaluated at x_w + r_j, times the wire window, real part, FFTG
// (usefulsubs.py:2245-2268).  Wire -> field: QW2Prop (qwoptics.py:717-805, without
// the plasmonic renormalisation) with the spline of each real-space wire source
// evaluated at x_j - x_w and summed over the wires; Rho = RhoH - RhoE
// (SBEs.py:5917).  The polarisation current J = (P^{n+1} - P^n) / dt drives the
// E update; Ex is the longitudinal field of Rho and Px (rhoPJ.py:703-880).
//
// Splines on the GPU.  The FMM spline is a tridiagonal solve whose elimination
// factors depend on the knots only; they are computed once.  The per-step
// forward and backward sweeps are first-order linear recurrences whose
// multipliers have magnitude ~2 - sqrt(3) = 0.268 on a uniform grid, so each
// thread solves a segment of kSeg points after kWarm warm-up points started from
// zero (0.268^48 ~ 3e-28 relative); the first and last segments start from the
// exact boundary values.
#include <cmath>
#include <vector>

#include "fp_bits.cuh"
#include "pstd.cuh"
#include "pstd3d.cuh"

namespace {
constexpr int kSeg = 16;
constexpr int kWarm = 48;
}  // namespace

struct SbeCouple {
  SbeCtx* ctx = nullptr;
  SbePstd* p = nullptr;
  int nw = 0, nprob_w = 0;
  long long tot_r = 0;
  SbeCoupleDesc desc{};
  double eta = 0.0;
  void* arena = nullptr;
  double* wx = nullptr;       // nw wire positions
  long long* probl = nullptr; // wire spline problems (5 per wire): knot offset, value offset
  int* probn = nullptr;       // knots per problem
  long long* wfl = nullptr;   // per-wire knot sets (2 per wire: offset, 0)
  int* wfn = nullptr;         // knots per wire
  double *g_b = nullptr, *g_t = nullptr;   // grid pivots and multipliers (nx)
  double *w_b = nullptr, *w_t = nullptr;   // wire-grid pivots and multipliers (tot_r)
  double2 *g_y = nullptr, *g_c1 = nullptr, *g_c2 = nullptr, *g_coef = nullptr;
  double2 *w_c1 = nullptr, *w_c2 = nullptr, *w_coef = nullptr;
  double2* twr = nullptr;     // tot_r: exp(-2 pi i m / Nr) per wire
  float2* twrf = nullptr;     // the same in FP32
  double2* wv = nullptr;      // 3 tot_r: sampled fields on the wire grids (real parts)
  float* wvf = nullptr;       // the same in FP32
  double2 *Ek = nullptr, *dEk = nullptr, *src = nullptr;  // 3, 3, 5 x tot_r
  double2 *Pg = nullptr, *Pold = nullptr, *rho = nullptr, *J = nullptr;  // 3, 3, 1, 2 x nx
  long long* step = nullptr;  // device step counter
};

namespace sbe {
namespace {

// ---- spline pieces ----------------------------------------------------------
struct SplBatch {
  const double* X;      // knots base
  const double* B;      // pivots base (indexed like X)
  const double* T;      // multipliers base
  const double2* Y;     // values base
  double2* C1;          // scratch (indexed like Y)
  double2* C2;
  double2* coef;        // 3 per value: b, c, d blocks of n
  const int* n;         // per problem (nullptr: n0 for all)
  const long long* off; // per problem: ko, vo (nullptr: ko = 0, vo = p * n0)
  int n0;
};

__device__ __forceinline__ void prob_of(const SplBatch& s, int p, int& n, long long& ko,
                                        long long& vo) {
  if (s.off) {
    n = s.n[p];
    ko = s.off[2 * p];
    vo = s.off[2 * p + 1];
  } else {
    n = s.n0;
    ko = 0;
    vo = (long long)p * s.n0;
  }
}

// numpy complex / complex with a zero imaginary divisor: a * (1 / d).
__device__ __forceinline__ double2 cdivr(double2 a, double d) {
  const double s = 1.0 / d;
  return make_double2(a.x * s, a.y * s);
}

// Pivots b and multipliers t of the FMM forward elimination (spliner.py:1338-1373).
__global__ void k_spl_factors(int nprob, const double* X, const int* nv, const long long* off,
                              int n0, double* B, double* T) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const int n = nv ? nv[p] : n0;
  const long long ko = off ? off[2 * p] : 0;
  const double* x = X + ko;
  double* b = B + ko;
  double* t = T + ko;
  for (int i = 1; i < n - 1; ++i) b[i] = 2.0 * ((x[i] - x[i - 1]) + (x[i + 1] - x[i]));
  b[0] = -(x[1] - x[0]);
  b[n - 1] = -(x[n - 1] - x[n - 2]);
  t[0] = 0.0;
  for (int i = 1; i < n; ++i) {
    const double d = x[i] - x[i - 1];
    t[i] = d * (1.0 / b[i - 1]);  // numpy complex division by (b + 0i)
    b[i] = b[i] - t[i] * d;
  }
}

__device__ __forceinline__ double2 delta(const double2* y, const double* x, int i) {
  return cdivr(csub(y[i + 1], y[i]), x[i + 1] - x[i]);
}

// Right-hand side: second differences and the FMM end conditions.
__global__ void k_spl_rhs(SplBatch s) {
  const int p = blockIdx.y;
  int n;
  long long ko, vo;
  prob_of(s, p, n, ko, vo);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* x = s.X + ko;
  const double2* y = s.Y + vo;
  double2 c;
  if (i >= 1 && i <= n - 2) {
    c = csub(delta(y, x, i), delta(y, x, i - 1));
  } else if (i == 0) {
    const double2 s1 = csub(delta(y, x, 1), delta(y, x, 0));
    const double2 s2 = csub(delta(y, x, 2), delta(y, x, 1));
    c = csub(cdivr(s2, x[3] - x[1]), cdivr(s1, x[2] - x[0]));
    const double d0 = x[1] - x[0];
    c = cdivr(cscale(c, d0 * d0), x[3] - x[0]);
  } else {
    const double2 sa = csub(delta(y, x, n - 2), delta(y, x, n - 3));
    const double2 sb = csub(delta(y, x, n - 3), delta(y, x, n - 4));
    c = csub(cdivr(sa, x[n - 1] - x[n - 3]), cdivr(sb, x[n - 2] - x[n - 4]));
    const double dl = x[n - 1] - x[n - 2];
    c = cdivr(cscale(make_double2(-c.x, -c.y), dl * dl), x[n - 1] - x[n - 4]);
  }
  s.C1[vo + i] = c;
}

// Forward sweep c_i -= t_i c_{i-1}, then c_{n-1} /= b_{n-1}.
__global__ void k_spl_fwd(SplBatch s) {
  const int p = blockIdx.y;
  int n;
  long long ko, vo;
  prob_of(s, p, n, ko, vo);
  const int s0 = (blockIdx.x * blockDim.x + threadIdx.x) * kSeg;
  if (s0 >= n) return;
  const double* t = s.T + ko;
  const double2* c1 = s.C1 + vo;
  double2* c2 = s.C2 + vo;
  const int e = min(s0 + kSeg, n);
  int i0 = max(1, s0 - kWarm);
  double2 v = (i0 == 1) ? c1[0] : make_double2(0.0, 0.0);
  if (s0 == 0) c2[0] = c1[0];
  for (int i = i0; i < e; ++i) {
    const double ti = t[i];
    const double2 ci = c1[i];
    v = make_double2(ci.x - ti * v.x, ci.y - ti * v.y);
    if (i >= s0) c2[i] = v;
  }
  if (e == n) c2[n - 1] = cdivr(v, s.B[ko + n - 1]);
}

// Backward sweep c_i = (c_i - d_i c_{i+1}) / b_i.
__global__ void k_spl_bwd(SplBatch s) {
  const int p = blockIdx.y;
  int n;
  long long ko, vo;
  prob_of(s, p, n, ko, vo);
  const int s0 = (blockIdx.x * blockDim.x + threadIdx.x) * kSeg;
  if (s0 >= n) return;
  const double* x = s.X + ko;
  const double* b = s.B + ko;
  const double2* c2 = s.C2 + vo;
  double2* c3 = s.C1 + vo;  // the right-hand side is dead: reuse its buffer
  const int e = min(s0 + kSeg, n);
  if (e == n) c3[n - 1] = c2[n - 1];
  const int i0 = min(n - 2, e - 1 + kWarm);
  double2 v = (i0 == n - 2) ? c2[n - 1] : make_double2(0.0, 0.0);
  for (int i = i0; i >= s0; --i) {
    const double di = x[i + 1] - x[i];
    const double2 ci = c2[i];
    v = cdivr(make_double2(ci.x - di * v.x, ci.y - di * v.y), b[i]);
    if (i < e) c3[i] = v;
  }
}

// Final coefficients (spliner.py:1384-1394).
__global__ void k_spl_final(SplBatch s) {
  const int p = blockIdx.y;
  int n;
  long long ko, vo;
  prob_of(s, p, n, ko, vo);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* x = s.X + ko;
  const double2* y = s.Y + vo;
  const double2* c = s.C1 + vo;
  double2* bb = s.coef + 3 * vo;
  double2* cc = bb + n;
  double2* dd = bb + 2 * n;
  if (i < n - 1) {
    const double di = x[i + 1] - x[i];
    const double2 t = cadd(c[i + 1], cscale(c[i], 2.0));
    bb[i] = csub(cdivr(csub(y[i + 1], y[i]), di), cscale(t, di));
    dd[i] = cdivr(csub(c[i + 1], c[i]), di);
    cc[i] = cscale(c[i], 3.0);
  } else {
    const double dl = x[n - 1] - x[n - 2];
    const double2 t = cadd(c[n - 2], cscale(c[n - 1], 2.0));
    bb[i] = cadd(cdivr(csub(y[n - 1], y[n - 2]), dl), cscale(t, dl));
    cc[i] = cscale(c[n - 1], 3.0);
    dd[i] = cdivr(csub(c[n - 1], c[n - 2]), dl);
  }
}

__device__ __forceinline__ int locate_sorted(const double* xx, int n, double x) {
  if (x < xx[0]) return 0;
  if (x >= xx[n - 1]) return n - 1;
  int jl = 0, ju = n;
  while (ju - jl > 1) {
    const int jm = (ju + jl) >> 1;
    if (x >= xx[jm]) jl = jm;
    else ju = jm;
  }
  return jl;
}

__device__ __forceinline__ double2 spl_eval(const double2* y, const double2* b, int n, int i,
                                            double dx) {
  const double2* c = b + n;
  const double2* d = b + 2 * n;
  double2 t = cadd(c[i], cscale(d[i], dx));
  t = cadd(b[i], cscale(t, dx));
  return cadd(y[i], cscale(t, dx));
}

// Grid fields -> wire grids: spline at x_w + r_j, window, real part.
__global__ void k_couple_eval(const WireDev* wires, int nx, const double* xg, const double2* gy,
                              const double2* gcoef, const double* wx, const double* r,
                              const double* window, double2* wv, float* wvf) {
  const int w = blockIdx.y;
  const WireDev W = wires[w];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= W.nr) return;
  const double u = wx[w] + r[W.off_r + j];
  const double win = window[W.off_r + j];
  double v[3] = {0.0, 0.0, 0.0};
  if (u >= xg[0] && u <= xg[nx - 1]) {
    const int i = locate_sorted(xg, nx, u);
    const double dx = u - xg[i];
    for (int f = 0; f < 3; ++f)
      v[f] = spl_eval(gy + (long long)f * nx, gcoef + 3LL * f * nx, nx, i, dx).x;
  }
  for (int f = 0; f < 3; ++f) {
    const double a = v[f] * win;
    wv[3 * W.off_r + (long long)f * W.nr + j] = make_double2(a, 0.0);
    wvf[3 * W.off_r + (long long)f * W.nr + j] = f64_to_f32(a);
  }
}

// FFTG as k_couple_fftg in FP32 with compensated (Kahan) sums, for the
// mixed-precision step (its field operands are FP32 values).  The sampled fields are
// real, so Ek[Nr - q] = conj(Ek[q]): the warps sum q = 0 .. Nr / 2 (Nr = 2 Nk + 2 is
// even) and store both.
__global__ void __launch_bounds__(256) k_couple_fftg_f(const WireDev* wires, const float2* twr,
                                                       const float* wv, double2* Ek) {
  const int w = blockIdx.y;
  const WireDev W = wires[w];
  const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (2 * q > W.nr) return;
  const int nr = W.nr;
  const float2* tw = twr + W.off_r;
  const float* v0 = wv + 3 * W.off_r;
  float s[6] = {0, 0, 0, 0, 0, 0}, cmp[6] = {0, 0, 0, 0, 0, 0};
  int m = (int)(((long long)q * lane) % nr);
  const int step = (int)(((long long)q * 32) % nr);
  for (int j = lane; j < nr; j += 32) {
    const float2 t = tw[m];
    for (int f = 0; f < 3; ++f) {
      const float a = v0[(long long)f * nr + j];
      const float terms[2] = {a * t.x, a * t.y};
      for (int c = 0; c < 2; ++c) {
        const int i = 2 * f + c;
        const float y = terms[c] - cmp[i];
        const float tt = s[i] + y;
        cmp[i] = (tt - s[i]) - y;
        s[i] = tt;
      }
    }
    m += step;
    if (m >= nr) m -= nr;
  }
  for (int i = 0; i < 6; ++i) {
    s[i] -= cmp[i];
    for (int o = 16; o > 0; o >>= 1) s[i] += __shfl_xor_sync(0xffffffffu, s[i], o);
  }
  if (lane == 0)
    for (int f = 0; f < 3; ++f) {
      const double re = -f32_to_f64(s[2 * f]) / nr, im = -f32_to_f64(s[2 * f + 1]) / nr;
      double2* e = Ek + 3 * W.off_r + (long long)f * nr;
      e[q] = make_double2(re, im);
      if (q > 0 && 2 * q < nr) e[nr - q] = make_double2(re, -im);
    }
}

// FFTG of the three sampled fields of every wire: Ek[q] = -(1/Nr) sum_j v_j e^{-2 pi i q j/Nr}.
// One warp per q; the twiddle table holds exp(-2 pi i m / Nr).
__global__ void __launch_bounds__(256) k_couple_fftg(const WireDev* wires, const double2* twr,
                                                     const double2* wv, double2* Ek) {
  const int w = blockIdx.y;
  const WireDev W = wires[w];
  const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= W.nr) return;
  const int nr = W.nr;
  const double2* tw = twr + W.off_r;
  const double2* v0 = wv + 3 * W.off_r;
  double sr[3] = {0, 0, 0}, si[3] = {0, 0, 0};
  int m = (int)(((long long)q * lane) % nr);
  const int step = (int)(((long long)q * 32) % nr);
  for (int j = lane; j < nr; j += 32) {
    const double2 t = tw[m];
    for (int f = 0; f < 3; ++f) {
      const double a = v0[(long long)f * nr + j].x;
      sr[f] = fma(a, t.x, sr[f]);
      si[f] = fma(a, t.y, si[f]);
    }
    m += step;
    if (m >= nr) m -= nr;
  }
  for (int f = 0; f < 3; ++f) {
    for (int o = 16; o > 0; o >>= 1) {
      sr[f] += __shfl_xor_sync(0xffffffffu, sr[f], o);
      si[f] += __shfl_xor_sync(0xffffffffu, si[f], o);
    }
  }
  if (lane == 0)
    for (int f = 0; f < 3; ++f)
      Ek[3 * W.off_r + (long long)f * nr + q] = make_double2(-sr[f] / nr, -si[f] / nr);
}

// Wire sources -> grid: spline of each wire's (Px, Py, Pz, re, rh) at x_j - x_w,
// summed over the wires; rho = sum_w (rh_w - re_w).
// The wires' positions and grid ends are staged in shared memory DEP_CHUNK wires at a
// time, so that the test of a wire against the grid point costs no global load; the
// wires are added in index order as before.
constexpr int DEP_CHUNK = 256;

__global__ void __launch_bounds__(64) k_couple_deposit(const WireDev* wires, int nw, int nx,
                                                       const double* xg, const double* wx,
                                                       const double* r, const double2* src,
                                                       const double2* wcoef, double2* Pg,
                                                       double2* rho) {
  __shared__ double s_wx[DEP_CHUNK], s_r0[DEP_CHUNK], s_r1[DEP_CHUNK];
  __shared__ long long s_off[DEP_CHUNK];
  __shared__ int s_nr[DEP_CHUNK];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = j < nx;
  double2 P[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  double2 rh = make_double2(0, 0);
  const double xj = in ? xg[j] : 0.0;
  for (int w0 = 0; w0 < nw; w0 += DEP_CHUNK) {
    const int nc = min(DEP_CHUNK, nw - w0);
    __syncthreads();   // the previous chunk is no longer read
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
      const WireDev& W = wires[w0 + i];
      s_wx[i] = wx[w0 + i];
      s_r0[i] = r[W.off_r];
      s_r1[i] = r[W.off_r + W.nr - 1];
      s_off[i] = W.off_r;
      s_nr[i] = W.nr;
    }
    __syncthreads();
    if (!in) continue;
    for (int k = 0; k < nc; ++k) {
      const double u = xj - s_wx[k];
      if (!(u >= s_r0[k] && u <= s_r1[k])) continue;
      const long long off = s_off[k];
      const int nr = s_nr[k];
      const double* rw = r + off;
      const int i = locate_sorted(rw, nr, u);
      const double dx = u - rw[i];
      const double2* y = src + 5 * off;
      const double2* cf = wcoef + 15 * off;
      double2 v[5];
      for (int c = 0; c < 5; ++c) v[c] = spl_eval(y + (long long)c * nr, cf + 3LL * c * nr, nr, i, dx);
      for (int c = 0; c < 3; ++c) P[c] = cadd(P[c], v[c]);
      rh = cadd(rh, csub(v[4], v[3]));
    }
  }
  if (!in) return;
  for (int c = 0; c < 3; ++c) Pg[(long long)c * nx + j] = P[c];
  rho[j] = rh;
}

// J = (P^{n+1} - P^n)/dt (y, z) plus the soft source; P^n <- P^{n+1}.
__global__ void k_couple_current(int nx, double dt, const double2* Pg, double2* Pold, double2* J,
                                 const long long* step, double t0, int src_index, double jamp,
                                 double tau, double w0, double tpeak) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nx) return;
  for (int c = 0; c < 3; ++c) {
    const double2 pn = Pg[(long long)c * nx + j];
    if (c > 0) {
      const double2 po = Pold[(long long)c * nx + j];
      J[(long long)(c - 1) * nx + j] = make_double2((pn.x - po.x) / dt, (pn.y - po.y) / dt);
    }
    Pold[(long long)c * nx + j] = pn;
  }
  if (j == src_index) {
    const double th = t0 + ((double)(*step) + 0.5) * dt;
    const double a = (th - tpeak) / tau;
    const double einc = exp(-a * a) * cos(w0 * (th - tpeak));
    J[j].x += jamp * einc;
  }
}

__global__ void k_tick(long long* step) { *step += 1; }

__global__ void k_stage3(int nx, const double2* Ex, const double2* E, double2* gy) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nx) return;
  gy[j] = Ex[j];
  gy[nx + j] = E[j];
  gy[2LL * nx + j] = E[nx + j];
}

__global__ void k_twr(const WireDev* wires, double2* twr, float2* twrf) {
  const int w = blockIdx.y;
  const WireDev W = wires[w];
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= W.nr) return;
  double s, c;
  sincospi(-2.0 * (double)m / (double)W.nr, &s, &c);
  twr[W.off_r + m] = make_double2(c, s);
  twrf[W.off_r + m] = make_float2(f64_to_f32(c), f64_to_f32(s));
}

void run_splines(const SplBatch& b, int nprob, int nmax, cudaStream_t s) {
  const int tpb = 128;
  const dim3 ge((nmax + tpb - 1) / tpb, nprob);
  const int nseg = (nmax + kSeg - 1) / kSeg;
  const dim3 gs((nseg + tpb - 1) / tpb, nprob);
  k_spl_rhs<<<ge, tpb, 0, s>>>(b);
  k_spl_fwd<<<gs, tpb, 0, s>>>(b);
  k_spl_bwd<<<gs, tpb, 0, s>>>(b);
  k_spl_final<<<ge, tpb, 0, s>>>(b);
}

SplBatch grid_batch(SbeCouple* cp) {
  SplBatch b{};
  b.X = cp->p->x;
  b.B = cp->g_b;
  b.T = cp->g_t;
  b.Y = cp->g_y;
  b.C1 = cp->g_c1;
  b.C2 = cp->g_c2;
  b.coef = cp->g_coef;
  b.n0 = cp->p->nx;
  return b;
}

SplBatch wire_batch(SbeCouple* cp) {
  SplBatch b{};
  b.X = cp->ctx->r;
  b.B = cp->w_b;
  b.T = cp->w_t;
  b.Y = cp->src;
  b.C1 = cp->w_c1;
  b.C2 = cp->w_c2;
  b.coef = cp->w_coef;
  b.n = cp->probn;
  b.off = cp->probl;
  return b;
}

// ---- wires along z on the 3-D grid --------------------------------------------
// Wire w lies along the grid's z axis at (x_w, y_w), centred at z = 0; its own axis
// is the reference wire's x, so the wire's field components (x, y, z) are the grid's
// (Ez, Ex, Ey) and its sources (Px, Py, Pz) go to the grid's (Pz, Px, Py).

// The three grid fields on the line of each wire (bilinear in x, y at every grid z):
// lines[w][f][k], f the wire's component.
__global__ void k_c3_lines(int nx, int ny, int nz, const double* xg, const double* yg,
                           const double* wxy, const double2* E, double2* lines) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, w = blockIdx.y;
  if (k >= nz) return;
  const double xw = wxy[2 * w], yw = wxy[2 * w + 1];
  const int i0 = min(max(locate_sorted(xg, nx, xw), 0), nx - 2);
  const int j0 = min(max(locate_sorted(yg, ny, yw), 0), ny - 2);
  const double fx = (xw - xg[i0]) / (xg[i0 + 1] - xg[i0]);
  const double fy = (yw - yg[j0]) / (yg[j0 + 1] - yg[j0]);
  const long long N = (long long)nx * ny * nz;
  const int src[3] = {2, 0, 1};   // wire x, y, z <- grid Ez, Ex, Ey
  for (int f = 0; f < 3; ++f) {
    const double2* F = E + src[f] * N;
    auto at = [&](int i, int j) { return F[((long long)i * ny + j) * nz + k]; };
    const double2 a = at(i0, j0), b = at(i0 + 1, j0), c = at(i0, j0 + 1), d = at(i0 + 1, j0 + 1);
    const double w00 = (1 - fx) * (1 - fy), w10 = fx * (1 - fy), w01 = (1 - fx) * fy, w11 = fx * fy;
    lines[((long long)w * 3 + f) * nz + k] =
        make_double2(w00 * a.x + w10 * b.x + w01 * c.x + w11 * d.x,
                     w00 * a.y + w10 * b.y + w01 * c.y + w11 * d.y);
  }
}

// Line splines -> wire grids: spline at z = r_j, window, real part.
__global__ void k_c3_eval(const WireDev* wires, int nz, const double* zg, const double2* lines,
                          const double2* lcoef, const double* r, const double* window, double2* wv,
                          float* wvf) {
  const int w = blockIdx.y;
  const WireDev W = wires[w];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= W.nr) return;
  const double u = r[W.off_r + j];
  const double win = window[W.off_r + j];
  double v[3] = {0.0, 0.0, 0.0};
  if (u >= zg[0] && u <= zg[nz - 1]) {
    const int i = locate_sorted(zg, nz, u);
    const double dz = u - zg[i];
    for (int f = 0; f < 3; ++f) {
      const long long pb = (long long)w * 3 + f;
      v[f] = spl_eval(lines + pb * nz, lcoef + 3 * pb * nz, nz, i, dz).x;
    }
  }
  for (int f = 0; f < 3; ++f) {
    const double a = v[f] * win;
    wv[3 * W.off_r + (long long)f * W.nr + j] = make_double2(a, 0.0);
    wvf[3 * W.off_r + (long long)f * W.nr + j] = f64_to_f32(a);
  }
}

// Wire sources on the grid z of their line: dl[w][c][k] for the grid components
// c = 0, 1, 2 (Px, Py, Pz of the grid) and 3 (rho = rh - re).
__global__ void k_c3_wire_lines(const WireDev* wires, int nz, const double* zg, const double* r,
                                const double2* src, const double2* wcoef, double2* dl) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, w = blockIdx.y;
  if (k >= nz) return;
  const WireDev W = wires[w];
  const double* rw = r + W.off_r;
  const double u = zg[k];
  double2 v[5];
  for (int c = 0; c < 5; ++c) v[c] = make_double2(0.0, 0.0);
  if (u >= rw[0] && u <= rw[W.nr - 1]) {
    const int i = locate_sorted(rw, W.nr, u);
    const double dx = u - rw[i];
    const double2* y = src + 5 * W.off_r;
    const double2* cf = wcoef + 15 * W.off_r;
    for (int c = 0; c < 5; ++c)
      v[c] = spl_eval(y + (long long)c * W.nr, cf + 3LL * c * W.nr, W.nr, i, dx);
  }
  double2* o = dl + (long long)w * 4 * nz;
  o[k] = v[1];            // grid Px <- wire Py
  o[nz + k] = v[2];       // grid Py <- wire Pz
  o[2 * nz + k] = v[0];   // grid Pz <- wire Px (along the wire)
  o[3 * nz + k] = csub(v[4], v[3]);
}

// Grid polarisation of the wires' gated lines, the current J = (P^{n+1} - P^n)/dt
// (P^n <- P^{n+1}), rho, and the soft source: a current sheet in the plane
// x = x[src_index] along component pol with the profile exp(-(y^2 + z^2)/waist^2).
// One block per (x, y) column, threads along z; the column's wires and gate weights
// come from a list built at creation.
struct C3Dep {
  int nx, ny, nz;
  const int* col_start;   // nx ny + 1
  const int* col_wire;
  const double* col_gate;
  const double2* dl;      // [w][4][nz]
  double2* Pold;          // 3 N
  double2* J;             // 3 N
  double2* rho;           // N
  double dt;
  // source
  const long long* step;
  double t0, jamp, tau, w0, tpeak, waist;
  int src_index, pol;
  const double* yg;
  const double* zg;
};

__global__ void k_c3_deposit(C3Dep a) {
  const int col = blockIdx.x;
  const int i = col / a.ny, j = col % a.ny;
  const long long N = (long long)a.nx * a.ny * a.nz;
  const int b = a.col_start[col], e = a.col_start[col + 1];
  double src_amp = 0.0;
  if (i == a.src_index) {
    const double th = a.t0 + ((double)(*a.step) + 0.5) * a.dt;
    const double u = (th - a.tpeak) / a.tau;
    src_amp = a.jamp * exp(-u * u) * cos(a.w0 * (th - a.tpeak));
  }
  for (int k = threadIdx.x; k < a.nz; k += blockDim.x) {
    double2 P[4] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0),
                    make_double2(0, 0)};
    for (int q = b; q < e; ++q) {
      const double g = a.col_gate[q];
      const double2* l = a.dl + (long long)a.col_wire[q] * 4 * a.nz;
      for (int c = 0; c < 4; ++c) {
        const double2 v = l[(long long)c * a.nz + k];
        P[c].x += g * v.x;
        P[c].y += g * v.y;
      }
    }
    const long long g0 = (long long)col * a.nz + k;
    for (int c = 0; c < 3; ++c) {
      const double2 po = a.Pold[c * N + g0];
      double2 jj = make_double2((P[c].x - po.x) / a.dt, (P[c].y - po.y) / a.dt);
      if (c == a.pol && src_amp != 0.0) {
        double prof = 1.0;
        if (a.waist > 0.0) {
          const double y = a.yg[j], z = a.zg[k];
          prof = exp(-(y * y + z * z) / (a.waist * a.waist));
        }
        jj.x += src_amp * prof;
      }
      a.J[c * N + g0] = jj;
      a.Pold[c * N + g0] = P[c];
    }
    a.rho[g0] = P[3];
  }
}

}  // namespace

int couple_sample(SbeCouple* cp, const double2* Ex, const double2* E, int precision,
                  cudaStream_t s) {
  SbeCtx* c = cp->ctx;
  const int nx = cp->p->nx;
  k_stage3<<<(nx + 255) / 256, 256, 0, s>>>(nx, Ex, E, cp->g_y);
  run_splines(grid_batch(cp), 3, nx, s);
  k_couple_eval<<<dim3((c->nr_max + 127) / 128, c->nw), 128, 0, s>>>(
      c->d_wires, nx, cp->p->x, cp->g_y, cp->g_coef, cp->wx, c->r, c->window, cp->wv, cp->wvf);
  if (precision == SBE_PREC_MIXED)
    k_couple_fftg_f<<<dim3((c->nr_max / 2 + 8) / 8, c->nw), 256, 0, s>>>(c->d_wires, cp->twrf,
                                                                         cp->wvf, cp->Ek);
  else
    k_couple_fftg<<<dim3((c->nr_max + 7) / 8, c->nw), 256, 0, s>>>(c->d_wires, cp->twr, cp->wv,
                                                                   cp->Ek);
  return cuda_check(cudaGetLastError(), "couple sample");
}

int couple_deposit(SbeCouple* cp, cudaStream_t s) {
  SbeCtx* c = cp->ctx;
  const int nx = cp->p->nx;
  run_splines(wire_batch(cp), cp->nprob_w, c->nr_max, s);
  k_couple_deposit<<<(nx + 63) / 64, 64, 0, s>>>(c->d_wires, c->nw, nx, cp->p->x, cp->wx, c->r,
                                                   cp->src, cp->w_coef, cp->Pg, cp->rho);
  return cuda_check(cudaGetLastError(), "couple deposit");
}

}  // namespace sbe

using namespace sbe;

namespace {
constexpr double kMu0c = 1.25663706127e-6;

int check_cp(SbeCouple* cp, const char* who) {
  if (!cp || !cp->ctx || !cp->p) return fail(SBE_ERR_ARG, std::string(who) + ": null coupling");
  return SBE_OK;
}
}  // namespace

extern "C" {

int sbe_couple_create(SbeCtx* c, SbePstd* p, const double* wire_x, const SbeCoupleDesc* d,
                      void* stream, SbeCouple** out) {
  if (!c || !p || !wire_x || !d || !out) return fail(SBE_ERR_ARG, "sbe_couple_create: null");
  *out = nullptr;
  if (d->src_index >= p->nx) return fail(SBE_ERR_ARG, "sbe_couple_create: source index outside grid");
  if (!(d->tau > 0.0) && d->src_index >= 0) return fail(SBE_ERR_ARG, "sbe_couple_create: tau <= 0");
  cudaStream_t s = as_stream(stream);
  SbeCouple* cp = new SbeCouple();
  cp->ctx = c;
  cp->p = p;
  cp->nw = c->nw;
  cp->tot_r = c->tot_r;
  cp->desc = *d;
  cp->eta = std::sqrt(kMu0c / (kEps0 * p->epsr));
  cp->nprob_w = 5 * c->nw;
  const long long nx = p->nx, R = c->tot_r;
  // arena layout (bytes, 256-aligned pieces)
  std::vector<std::pair<void**, size_t>> parts = {
      {(void**)&cp->wx, sizeof(double) * c->nw},
      {(void**)&cp->probn, sizeof(int) * cp->nprob_w},
      {(void**)&cp->probl, sizeof(long long) * 2 * cp->nprob_w},
      {(void**)&cp->wfn, sizeof(int) * c->nw},
      {(void**)&cp->wfl, sizeof(long long) * 2 * c->nw},
      {(void**)&cp->g_b, sizeof(double) * nx},
      {(void**)&cp->g_t, sizeof(double) * nx},
      {(void**)&cp->w_b, sizeof(double) * R},
      {(void**)&cp->w_t, sizeof(double) * R},
      {(void**)&cp->g_y, sizeof(double2) * 3 * nx},
      {(void**)&cp->g_c1, sizeof(double2) * 3 * nx},
      {(void**)&cp->g_c2, sizeof(double2) * 3 * nx},
      {(void**)&cp->g_coef, sizeof(double2) * 9 * nx},
      {(void**)&cp->w_c1, sizeof(double2) * 5 * R},
      {(void**)&cp->w_c2, sizeof(double2) * 5 * R},
      {(void**)&cp->w_coef, sizeof(double2) * 15 * R},
      {(void**)&cp->twr, sizeof(double2) * R},
      {(void**)&cp->twrf, sizeof(float2) * R},
      {(void**)&cp->wv, sizeof(double2) * 3 * R},
      {(void**)&cp->wvf, sizeof(float) * 3 * R},
      {(void**)&cp->Ek, sizeof(double2) * 3 * R},
      {(void**)&cp->dEk, sizeof(double2) * 3 * R},
      {(void**)&cp->src, sizeof(double2) * 5 * R},
      {(void**)&cp->Pg, sizeof(double2) * 3 * nx},
      {(void**)&cp->Pold, sizeof(double2) * 3 * nx},
      {(void**)&cp->rho, sizeof(double2) * nx},
      {(void**)&cp->J, sizeof(double2) * 2 * nx},
      {(void**)&cp->step, sizeof(long long)},
  };
  size_t total = 0;
  for (auto& pr : parts) total += (pr.second + 255) / 256 * 256;
  if (cudaMalloc(&cp->arena, total) != cudaSuccess) {
    delete cp;
    return fail(SBE_ERR_OOM, "sbe_couple_create: device allocation");
  }
  size_t o = 0;
  for (auto& pr : parts) {
    *pr.first = static_cast<char*>(cp->arena) + o;
    o += (pr.second + 255) / 256 * 256;
  }
  cudaMemsetAsync(cp->arena, 0, total, s);
  // wire spline problems: wire w, component k -> n = Nr, knots at off_r, values at 5 off_r + k Nr
  std::vector<int> pn(cp->nprob_w);
  std::vector<long long> pl(2 * cp->nprob_w);
  std::vector<long long> wl(2 * c->nw);
  std::vector<int> wn(c->nw);
  for (int w = 0; w < c->nw; ++w) {
    const WireDev& W = c->wires[w];
    wl[2 * w] = W.off_r;
    wl[2 * w + 1] = 0;
    wn[w] = W.nr;
    for (int k = 0; k < 5; ++k) {
      const int pi = 5 * w + k;
      pn[pi] = W.nr;
      pl[2 * pi] = W.off_r;
      pl[2 * pi + 1] = 5 * W.off_r + (long long)k * W.nr;
    }
  }
  cudaMemcpyAsync(cp->wx, wire_x, sizeof(double) * c->nw, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->probn, pn.data(), sizeof(int) * pn.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->probl, pl.data(), sizeof(long long) * pl.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->wfn, wn.data(), sizeof(int) * wn.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->wfl, wl.data(), sizeof(long long) * wl.size(), cudaMemcpyHostToDevice, s);
  // elimination factors of the grid knots and of each wire's knots (computed once)
  k_spl_factors<<<1, 32, 0, s>>>(1, p->x, nullptr, nullptr, p->nx, cp->g_b, cp->g_t);
  k_spl_factors<<<(c->nw + 31) / 32, 32, 0, s>>>(c->nw, c->r, cp->wfn, cp->wfl, 0, cp->w_b,
                                                 cp->w_t);
  k_twr<<<dim3((c->nr_max + 127) / 128, c->nw), 128, 0, s>>>(c->d_wires, cp->twr, cp->twrf);
  int rc = cuda_check(cudaGetLastError(), "sbe_couple_create");
  if (rc == SBE_OK) rc = cuda_check(cudaStreamSynchronize(s), "sbe_couple_create: tables");
  if (rc) {
    cudaFree(cp->arena);
    delete cp;
    return rc;
  }
  *out = cp;
  return SBE_OK;
}

int sbe_couple_destroy(SbeCouple* cp) {
  if (!cp) return SBE_OK;
  cudaFree(cp->arena);
  delete cp;
  return SBE_OK;
}

int sbe_couple_buffers(SbeCouple* cp, double** Ek, double** src, double** Pg, double** rho,
                       double** J) {
  int rc = check_cp(cp, "sbe_couple_buffers");
  if (rc) return rc;
  if (Ek) *Ek = reinterpret_cast<double*>(cp->Ek);
  if (src) *src = reinterpret_cast<double*>(cp->src);
  if (Pg) *Pg = reinterpret_cast<double*>(cp->Pg);
  if (rho) *rho = reinterpret_cast<double*>(cp->rho);
  if (J) *J = reinterpret_cast<double*>(cp->J);
  return SBE_OK;
}

int sbe_couple_set_step(SbeCouple* cp, long long n, void* stream) {
  int rc = check_cp(cp, "sbe_couple_set_step");
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);
  cudaMemcpyAsync(cp->step, &n, sizeof(long long), cudaMemcpyHostToDevice, s);
  return cuda_check(cudaStreamSynchronize(s), "sbe_couple_set_step");
}

int sbe_couple_reset(SbeCouple* cp, void* stream) {
  int rc = check_cp(cp, "sbe_couple_reset");
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);
  const size_t nx = cp->p->nx;
  cudaMemsetAsync(cp->Pg, 0, sizeof(double2) * 3 * nx, s);
  cudaMemsetAsync(cp->Pold, 0, sizeof(double2) * 3 * nx, s);
  cudaMemsetAsync(cp->rho, 0, sizeof(double2) * nx, s);
  cudaMemsetAsync(cp->J, 0, sizeof(double2) * 2 * nx, s);
  cudaMemsetAsync(cp->step, 0, sizeof(long long), s);
  return cuda_check(cudaGetLastError(), "sbe_couple_reset");
}

int sbe_couple_sample(SbeCouple* cp, const double* Ex, const double* E, void* stream) {
  int rc = check_cp(cp, "sbe_couple_sample");
  if (rc) return rc;
  if (!Ex || !E) return fail(SBE_ERR_ARG, "sbe_couple_sample: null field");
  return couple_sample(cp, reinterpret_cast<const double2*>(Ex),
                       reinterpret_cast<const double2*>(E), SBE_PREC_FP64, as_stream(stream));
}

int sbe_couple_deposit(SbeCouple* cp, void* stream) {
  int rc = check_cp(cp, "sbe_couple_deposit");
  if (rc) return rc;
  return couple_deposit(cp, as_stream(stream));
}

int sbe_couple_step(SbeCouple* cp, double* P, double* C, double* D, double* E, double* H,
                    double* Ex, double dt, int precision, void* stream) {
  int rc = check_cp(cp, "sbe_couple_step");
  if (rc) return rc;
  if (!P || !C || !D || !E || !H || !Ex) return fail(SBE_ERR_ARG, "sbe_couple_step: null");
  cudaStream_t s = as_stream(stream);
  SbePstd* p = cp->p;
  const int nx = p->nx;
  // 1. fields at t_n on the wires
  if ((rc = couple_sample(cp, reinterpret_cast<double2*>(Ex), reinterpret_cast<double2*>(E),
                          precision, s)))
    return rc;
  // 2. H^{n+1/2}
  if ((rc = sbe_pstd_update_h(p, E, H, dt, stream))) return rc;
  // 3. wires t_n -> t_{n+1} at the sampled field
  if ((rc = sbe_rk4_step(cp->ctx, P, C, D, reinterpret_cast<double*>(cp->Ek),
                         reinterpret_cast<double*>(cp->dEk), dt, precision,
                         reinterpret_cast<double*>(cp->src), stream)))
    return rc;
  // 4. sources on the grid, current, E^{n+1}
  if ((rc = couple_deposit(cp, s))) return rc;
  const SbeCoupleDesc& d = cp->desc;
  const double jamp = d.src_index >= 0 ? -2.0 * d.E0 / (cp->eta * p->dx) : 0.0;
  k_couple_current<<<(nx + 255) / 256, 256, 0, s>>>(nx, dt, cp->Pg, cp->Pold, cp->J, cp->step,
                                                    d.t0, d.src_index, jamp, d.tau, d.w0,
                                                    d.tpeak);
  if ((rc = cuda_check(cudaGetLastError(), "couple current"))) return rc;
  if ((rc = sbe_pstd_update_e(p, E, H, reinterpret_cast<double*>(cp->J), dt, stream))) return rc;
  // 5. longitudinal field of the new charge and Px
  if (d.longitudinal) {
    if ((rc = sbe_pstd_elong(p, reinterpret_cast<double*>(cp->rho),
                             reinterpret_cast<double*>(cp->Pg), Ex, stream)))
      return rc;
  }
  k_tick<<<1, 1, 0, s>>>(cp->step);
  return cuda_check(cudaGetLastError(), "sbe_couple_step");
}

int sbe_couple_graph_create(SbeCouple* cp, double* P, double* C, double* D, double* E, double* H,
                            double* Ex, double dt, int precision, SbeGraph** out,
                            long long* n_kernels) {
  int rc = check_cp(cp, "sbe_couple_graph_create");
  if (rc) return rc;
  if (!out) return fail(SBE_ERR_ARG, "sbe_couple_graph_create: null");
  return capture_graph(
      cp->ctx, precision,
      [&](cudaStream_t cs) { return sbe_couple_step(cp, P, C, D, E, H, Ex, dt, precision, (void*)cs); },
      out, n_kernels);
}

}  // extern "C"

// ---- wires along z on the 3-D grid ---------------------------------------------
struct SbeCouple3 {
  SbeCtx* ctx = nullptr;
  SbePstd3* p = nullptr;
  int nw = 0;
  SbeCouple3Desc desc{};
  double eta = 0.0;
  void* arena = nullptr;
  double* wxy = nullptr;        // 2 nw wire positions (x, y)
  int *col_start = nullptr, *col_wire = nullptr;
  double* col_gate = nullptr;
  int *probn = nullptr, *wfn = nullptr;
  long long *probl = nullptr, *wfl = nullptr;
  double *z_b = nullptr, *z_t = nullptr;   // spline factors of the grid z knots
  double *w_b = nullptr, *w_t = nullptr;   // of the wire knots
  double2 *lines = nullptr, *l_c1 = nullptr, *l_c2 = nullptr, *l_coef = nullptr;   // 3 nw nz
  double2 *w_c1 = nullptr, *w_c2 = nullptr, *w_coef = nullptr;
  double2* twr = nullptr;
  float2* twrf = nullptr;
  double2* wv = nullptr;
  float* wvf = nullptr;
  double2 *Ek = nullptr, *dEk = nullptr, *src = nullptr;
  double2* dl = nullptr;        // 4 nw nz: wire sources on their lines
  double2 *Pold = nullptr, *J = nullptr, *rho = nullptr;   // 3 N, 3 N, N
  long long* step = nullptr;
};

namespace {

SplBatch line_batch(SbeCouple3* cp) {
  SplBatch b{};
  b.X = cp->p->x[2];
  b.B = cp->z_b;
  b.T = cp->z_t;
  b.Y = cp->lines;
  b.C1 = cp->l_c1;
  b.C2 = cp->l_c2;
  b.coef = cp->l_coef;
  b.n0 = cp->p->n[2];
  return b;
}

SplBatch wire_batch3(SbeCouple3* cp) {
  SplBatch b{};
  b.X = cp->ctx->r;
  b.B = cp->w_b;
  b.T = cp->w_t;
  b.Y = cp->src;
  b.C1 = cp->w_c1;
  b.C2 = cp->w_c2;
  b.coef = cp->w_coef;
  b.n = cp->probn;
  b.off = cp->probl;
  return b;
}

int check_cp3(SbeCouple3* cp, const char* who) {
  if (!cp || !cp->ctx || !cp->p) return fail(SBE_ERR_ARG, std::string(who) + ": null coupling");
  return SBE_OK;
}

int c3_sample(SbeCouple3* cp, const double2* E, int precision, cudaStream_t s) {
  SbeCtx* c = cp->ctx;
  SbePstd3* p = cp->p;
  const int nz = p->n[2];
  k_c3_lines<<<dim3((nz + 127) / 128, c->nw), 128, 0, s>>>(p->n[0], p->n[1], nz, p->x[0],
                                                           p->x[1], cp->wxy, E, cp->lines);
  run_splines(line_batch(cp), 3 * c->nw, nz, s);
  k_c3_eval<<<dim3((c->nr_max + 127) / 128, c->nw), 128, 0, s>>>(
      c->d_wires, nz, p->x[2], cp->lines, cp->l_coef, c->r, c->window, cp->wv, cp->wvf);
  if (precision == SBE_PREC_MIXED)
    k_couple_fftg_f<<<dim3((c->nr_max / 2 + 8) / 8, c->nw), 256, 0, s>>>(c->d_wires, cp->twrf,
                                                                         cp->wvf, cp->Ek);
  else
    k_couple_fftg<<<dim3((c->nr_max + 7) / 8, c->nw), 256, 0, s>>>(c->d_wires, cp->twr, cp->wv,
                                                                   cp->Ek);
  return cuda_check(cudaGetLastError(), "couple3 sample");
}

int c3_deposit(SbeCouple3* cp, double dt, cudaStream_t s) {
  SbeCtx* c = cp->ctx;
  SbePstd3* p = cp->p;
  const int nz = p->n[2];
  run_splines(wire_batch3(cp), 5 * c->nw, c->nr_max, s);
  k_c3_wire_lines<<<dim3((nz + 127) / 128, c->nw), 128, 0, s>>>(c->d_wires, nz, p->x[2], c->r,
                                                                cp->src, cp->w_coef, cp->dl);
  C3Dep a{};
  a.nx = p->n[0];
  a.ny = p->n[1];
  a.nz = nz;
  a.col_start = cp->col_start;
  a.col_wire = cp->col_wire;
  a.col_gate = cp->col_gate;
  a.dl = cp->dl;
  a.Pold = cp->Pold;
  a.J = cp->J;
  a.rho = cp->rho;
  a.dt = dt;
  const SbeCouple3Desc& d = cp->desc;
  a.step = cp->step;
  a.t0 = d.t0;
  a.jamp = d.src_index >= 0 ? -2.0 * d.E0 / (cp->eta * p->d[0]) : 0.0;
  a.tau = d.tau;
  a.w0 = d.w0;
  a.tpeak = d.tpeak;
  a.waist = d.waist;
  a.src_index = d.src_index;
  a.pol = d.pol;
  a.yg = p->x[1];
  a.zg = p->x[2];
  k_c3_deposit<<<p->n[0] * p->n[1], 128, 0, s>>>(a);
  return cuda_check(cudaGetLastError(), "couple3 deposit");
}

}  // namespace

extern "C" {

int sbe_couple3_create(SbeCtx* c, SbePstd3* p, const double* wire_xy, const SbeCouple3Desc* d,
                       void* stream, SbeCouple3** out) {
  if (!c || !p || !wire_xy || !d || !out) return fail(SBE_ERR_ARG, "sbe_couple3_create: null");
  *out = nullptr;
  if (d->src_index >= p->n[0] || d->pol < 0 || d->pol > 2)
    return fail(SBE_ERR_ARG, "sbe_couple3_create: source plane or polarisation");
  if (d->src_index >= 0 && !(d->tau > 0.0)) return fail(SBE_ERR_ARG, "sbe_couple3_create: tau");
  if (!(d->gate > 0.0)) return fail(SBE_ERR_ARG, "sbe_couple3_create: gate length");
  const int nx = p->n[0], ny = p->n[1], nz = p->n[2];
  std::vector<double> xg(nx), yg(ny);
  cudaStream_t s = as_stream(stream);
  // the wires' gated columns: gate exp(-(x - x_w)^2 / (2 a^2)) exp(-(y - y_w)^2 / (2 a^2))
  // (the reference's SHO gates, rhoPJ.py:383-389), every column where it is nonzero
  int rc = cuda_check(cudaMemcpy(xg.data(), p->x[0], sizeof(double) * nx, cudaMemcpyDeviceToHost),
                      "sbe_couple3_create: grid");
  if (!rc) rc = cuda_check(cudaMemcpy(yg.data(), p->x[1], sizeof(double) * ny,
                                      cudaMemcpyDeviceToHost), "sbe_couple3_create: grid");
  if (rc) return rc;
  for (int w = 0; w < c->nw; ++w)
    if (!(wire_xy[2 * w] >= xg[0] && wire_xy[2 * w] <= xg[nx - 1] &&
          wire_xy[2 * w + 1] >= yg[0] && wire_xy[2 * w + 1] <= yg[ny - 1]))
      return fail(SBE_ERR_ARG, "sbe_couple3_create: wire outside the grid");
  const double a2 = 2.0 * d->gate * d->gate;
  std::vector<int> cstart(nx * ny + 1, 0), cwire;
  std::vector<double> cgate;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      cstart[i * ny + j] = (int)cwire.size();
      for (int w = 0; w < c->nw; ++w) {
        const double dx = xg[i] - wire_xy[2 * w], dy = yg[j] - wire_xy[2 * w + 1];
        const double g = std::exp(-dx * dx / a2) * std::exp(-dy * dy / a2);
        if (g > 0.0) {
          cwire.push_back(w);
          cgate.push_back(g);
        }
      }
    }
  cstart[nx * ny] = (int)cwire.size();
  SbeCouple3* cp = new SbeCouple3();
  cp->ctx = c;
  cp->p = p;
  cp->nw = c->nw;
  cp->desc = *d;
  cp->eta = std::sqrt(kMu0c / (kEps0 * p->epsr));
  const long long R = c->tot_r, N = p->N, L = 3LL * c->nw * nz;
  const int np = 5 * c->nw;
  std::vector<std::pair<void**, size_t>> parts = {
      {(void**)&cp->wxy, sizeof(double) * 2 * c->nw},
      {(void**)&cp->col_start, sizeof(int) * cstart.size()},
      {(void**)&cp->col_wire, sizeof(int) * std::max<size_t>(cwire.size(), 1)},
      {(void**)&cp->col_gate, sizeof(double) * std::max<size_t>(cgate.size(), 1)},
      {(void**)&cp->probn, sizeof(int) * np},
      {(void**)&cp->probl, sizeof(long long) * 2 * np},
      {(void**)&cp->wfn, sizeof(int) * c->nw},
      {(void**)&cp->wfl, sizeof(long long) * 2 * c->nw},
      {(void**)&cp->z_b, sizeof(double) * nz},
      {(void**)&cp->z_t, sizeof(double) * nz},
      {(void**)&cp->w_b, sizeof(double) * R},
      {(void**)&cp->w_t, sizeof(double) * R},
      {(void**)&cp->lines, sizeof(double2) * L},
      {(void**)&cp->l_c1, sizeof(double2) * L},
      {(void**)&cp->l_c2, sizeof(double2) * L},
      {(void**)&cp->l_coef, sizeof(double2) * 3 * L},
      {(void**)&cp->w_c1, sizeof(double2) * 5 * R},
      {(void**)&cp->w_c2, sizeof(double2) * 5 * R},
      {(void**)&cp->w_coef, sizeof(double2) * 15 * R},
      {(void**)&cp->twr, sizeof(double2) * R},
      {(void**)&cp->twrf, sizeof(float2) * R},
      {(void**)&cp->wv, sizeof(double2) * 3 * R},
      {(void**)&cp->wvf, sizeof(float) * 3 * R},
      {(void**)&cp->Ek, sizeof(double2) * 3 * R},
      {(void**)&cp->dEk, sizeof(double2) * 3 * R},
      {(void**)&cp->src, sizeof(double2) * 5 * R},
      {(void**)&cp->dl, sizeof(double2) * 4 * (size_t)c->nw * nz},
      {(void**)&cp->Pold, sizeof(double2) * 3 * N},
      {(void**)&cp->J, sizeof(double2) * 3 * N},
      {(void**)&cp->rho, sizeof(double2) * N},
      {(void**)&cp->step, sizeof(long long)},
  };
  size_t total = 0;
  for (auto& pr : parts) total += (pr.second + 255) / 256 * 256;
  if (cudaMalloc(&cp->arena, total) != cudaSuccess) {
    delete cp;
    return fail(SBE_ERR_OOM, "sbe_couple3_create: device allocation");
  }
  size_t o = 0;
  for (auto& pr : parts) {
    *pr.first = static_cast<char*>(cp->arena) + o;
    o += (pr.second + 255) / 256 * 256;
  }
  cudaMemsetAsync(cp->arena, 0, total, s);
  std::vector<int> pn(np);
  std::vector<long long> pl(2 * np), wl(2 * c->nw);
  std::vector<int> wn(c->nw);
  for (int w = 0; w < c->nw; ++w) {
    const WireDev& W = c->wires[w];
    wl[2 * w] = W.off_r;
    wl[2 * w + 1] = 0;
    wn[w] = W.nr;
    for (int k = 0; k < 5; ++k) {
      pn[5 * w + k] = W.nr;
      pl[2 * (5 * w + k)] = W.off_r;
      pl[2 * (5 * w + k) + 1] = 5 * W.off_r + (long long)k * W.nr;
    }
  }
  cudaMemcpyAsync(cp->wxy, wire_xy, sizeof(double) * 2 * c->nw, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->col_start, cstart.data(), sizeof(int) * cstart.size(),
                  cudaMemcpyHostToDevice, s);
  if (!cwire.empty()) {
    cudaMemcpyAsync(cp->col_wire, cwire.data(), sizeof(int) * cwire.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(cp->col_gate, cgate.data(), sizeof(double) * cgate.size(),
                    cudaMemcpyHostToDevice, s);
  }
  cudaMemcpyAsync(cp->probn, pn.data(), sizeof(int) * pn.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->probl, pl.data(), sizeof(long long) * pl.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->wfn, wn.data(), sizeof(int) * wn.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(cp->wfl, wl.data(), sizeof(long long) * wl.size(), cudaMemcpyHostToDevice, s);
  k_spl_factors<<<1, 32, 0, s>>>(1, p->x[2], nullptr, nullptr, nz, cp->z_b, cp->z_t);
  k_spl_factors<<<(c->nw + 31) / 32, 32, 0, s>>>(c->nw, c->r, cp->wfn, cp->wfl, 0, cp->w_b,
                                                 cp->w_t);
  k_twr<<<dim3((c->nr_max + 127) / 128, c->nw), 128, 0, s>>>(c->d_wires, cp->twr, cp->twrf);
  rc = cuda_check(cudaGetLastError(), "sbe_couple3_create");
  if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "sbe_couple3_create: tables");
  if (rc) {
    cudaFree(cp->arena);
    delete cp;
    return rc;
  }
  *out = cp;
  return SBE_OK;
}

int sbe_couple3_destroy(SbeCouple3* cp) {
  if (!cp) return SBE_OK;
  cudaFree(cp->arena);
  delete cp;
  return SBE_OK;
}

int sbe_couple3_buffers(SbeCouple3* cp, double** Ek, double** src, double** J, double** rho) {
  int rc = check_cp3(cp, "sbe_couple3_buffers");
  if (rc) return rc;
  if (Ek) *Ek = reinterpret_cast<double*>(cp->Ek);
  if (src) *src = reinterpret_cast<double*>(cp->src);
  if (J) *J = reinterpret_cast<double*>(cp->J);
  if (rho) *rho = reinterpret_cast<double*>(cp->rho);
  return SBE_OK;
}

int sbe_couple3_reset(SbeCouple3* cp, void* stream) {
  int rc = check_cp3(cp, "sbe_couple3_reset");
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);
  const size_t N = cp->p->N;
  cudaMemsetAsync(cp->Pold, 0, sizeof(double2) * 3 * N, s);
  cudaMemsetAsync(cp->J, 0, sizeof(double2) * 3 * N, s);
  cudaMemsetAsync(cp->rho, 0, sizeof(double2) * N, s);
  cudaMemsetAsync(cp->step, 0, sizeof(long long), s);
  return cuda_check(cudaGetLastError(), "sbe_couple3_reset");
}

int sbe_couple3_sample(SbeCouple3* cp, const double* E, int precision, void* stream) {
  int rc = check_cp3(cp, "sbe_couple3_sample");
  if (rc) return rc;
  if (!E) return fail(SBE_ERR_ARG, "sbe_couple3_sample: null field");
  return c3_sample(cp, reinterpret_cast<const double2*>(E), precision, as_stream(stream));
}

int sbe_couple3_deposit(SbeCouple3* cp, double dt, void* stream) {
  int rc = check_cp3(cp, "sbe_couple3_deposit");
  if (rc) return rc;
  return c3_deposit(cp, dt, as_stream(stream));
}

int sbe_couple3_step(SbeCouple3* cp, double* P, double* C, double* D, double* E, double* H,
                     double dt, int precision, void* stream) {
  int rc = check_cp3(cp, "sbe_couple3_step");
  if (rc) return rc;
  if (!P || !C || !D || !E || !H) return fail(SBE_ERR_ARG, "sbe_couple3_step: null");
  cudaStream_t s = as_stream(stream);
  if ((rc = c3_sample(cp, reinterpret_cast<const double2*>(E), precision, s))) return rc;
  // the H half-step leaves the transform of the new H for the E half-step (the wire
  // step and the deposit in between do not touch the field grid's work array)
  if ((rc = pstd3_update_h_fwd(cp->p, reinterpret_cast<const double2*>(E),
                               reinterpret_cast<double2*>(H), dt, s)))
    return rc;
  if ((rc = sbe_rk4_step(cp->ctx, P, C, D, reinterpret_cast<double*>(cp->Ek),
                         reinterpret_cast<double*>(cp->dEk), dt, precision,
                         reinterpret_cast<double*>(cp->src), stream)))
    return rc;
  if ((rc = c3_deposit(cp, dt, s))) return rc;
  if ((rc = pstd3_update_e_from_work(cp->p, reinterpret_cast<double2*>(E),
                                     reinterpret_cast<const double2*>(H), cp->J, dt, s)))
    return rc;
  k_tick<<<1, 1, 0, s>>>(cp->step);
  return cuda_check(cudaGetLastError(), "sbe_couple3_step");
}

int sbe_couple3_graph_create(SbeCouple3* cp, double* P, double* C, double* D, double* E,
                             double* H, double dt, int precision, SbeGraph** out,
                             long long* n_kernels) {
  int rc = check_cp3(cp, "sbe_couple3_graph_create");
  if (rc) return rc;
  if (!out) return fail(SBE_ERR_ARG, "sbe_couple3_graph_create: null");
  return capture_graph(
      cp->ctx, precision,
      [&](cudaStream_t cs) { return sbe_couple3_step(cp, P, C, D, E, H, dt, precision, (void*)cs); },
      out, n_kernels);
}

}  // extern "C"
