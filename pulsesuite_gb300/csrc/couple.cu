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
// mixed-precision step (its field operands are FP32 values).
__global__ void __launch_bounds__(256) k_couple_fftg_f(const WireDev* wires, const float2* twr,
                                                       const float* wv, double2* Ek) {
  const int w = blockIdx.y;
  const WireDev W = wires[w];
  const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= W.nr) return;
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
    for (int f = 0; f < 3; ++f)
      Ek[3 * W.off_r + (long long)f * nr + q] =
          make_double2(-f32_to_f64(s[2 * f]) / nr, -f32_to_f64(s[2 * f + 1]) / nr);
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
__global__ void k_couple_deposit(const WireDev* wires, int nw, int nx, const double* xg,
                                 const double* wx, const double* r, const double2* src,
                                 const double2* wcoef, double2* Pg, double2* rho) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nx) return;
  double2 P[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  double2 rh = make_double2(0, 0);
  const double xj = xg[j];
  for (int w = 0; w < nw; ++w) {
    const WireDev& W = wires[w];
    const double* rw = r + W.off_r;
    const double u = xj - wx[w];
    if (!(u >= rw[0] && u <= rw[W.nr - 1])) continue;
    const int i = locate_sorted(rw, W.nr, u);
    const double dx = u - rw[i];
    const double2* y = src + 5 * W.off_r;
    const double2* cf = wcoef + 15 * W.off_r;
    double2 v[5];
    for (int c = 0; c < 5; ++c)
      v[c] = spl_eval(y + (long long)c * W.nr, cf + 3LL * c * W.nr, W.nr, i, dx);
    for (int c = 0; c < 3; ++c) P[c] = cadd(P[c], v[c]);
    rh = cadd(rh, csub(v[4], v[3]));
  }
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
    k_couple_fftg_f<<<dim3((c->nr_max + 7) / 8, c->nw), 256, 0, s>>>(c->d_wires, cp->twrf,
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
  k_couple_deposit<<<(nx + 127) / 128, 128, 0, s>>>(c->d_wires, c->nw, nx, cp->p->x, cp->wx,
                                                     c->r, cp->src, cp->w_coef, cp->Pg, cp->rho);
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
