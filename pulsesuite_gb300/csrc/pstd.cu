// 1-D PSTD field step: spectral x-derivative by a four-step Stockham FFT in FP64
// with the k-space multiply and the field update fused into the passes.
//
// The reference has no 1-D Maxwell stepper; its pieces are the spectral derivative
// dfdx1D = IFFT(i q FFT f) (PSTD3D/usefulsubs.py:163-185), the grids of
// libpulsesuite/helpers.py:811-863, the longitudinal field of ElongfromRho
// (PSTD3D/rhoPJ.py:703-880) and the absorbing mask multiply of ApplyABC
// (usefulsubs.py:584-609).  The time step is the standard leapfrog
//   H^{n+1/2} = H^{n-1/2} - dt/mu0 curl E^n,  E^{n+1} = E^n + dt/eps (curl H^{n+1/2} - J^{n+1/2})
// for propagation along x: d_t Hz = -(1/mu0) d_x Ey, d_t Hy = (1/mu0) d_x Ez,
// d_t Ey = -(1/eps)(d_x Hz + Jy), d_t Ez = (1/eps)(d_x Hy - Jz).
//
// FFT of length nx = n1 n2 (n = n1' n2 + n2', k = k1 + n1 k2):
//   pass A  column FFTs of length n1 (stride n2), times exp(-2 pi i n2' k1 / nx)
//   pass B  row FFTs of length n2, k-space multiply, inverse row FFTs, times the
//           conjugate twiddle (one CTA holds whole rows, so the spectrum never
//           goes back to memory between the forward and inverse halves)
//   pass C  inverse column FFTs, 1/nx, and the field update.
// Each transform is a radix-2 Stockham sequence in shared memory; the field data
// crosses HBM/L2 three times per derivative.
#include <cmath>
#include <cstdio>

#include "pstd.cuh"

namespace sbe {
namespace {

constexpr double kMu0 = 1.25663706127e-6;  // CODATA 2022 (scipy.constants.mu_0)
constexpr int kCols = 8;                   // columns per CTA, passes A and C
constexpr int kRows = 8;                   // rows per CTA, pass B
constexpr int kThreads = 256;

__device__ __forceinline__ double2 ld(const double2* p) { return __ldg(p); }

// Radix-2 Stockham over shared memory.  ntr transforms of length L = 2^lg; element
// p of transform c lives at a[p * ps + c * cs].  rows_fast: consecutive threads walk
// p (transforms stored contiguously) instead of c.  dir -1: exp(-i ...), +1: exp(+i ...).
// Returns the buffer that holds the result (natural order).
__device__ double2* smem_fft(double2* a, double2* b, int lg, int lgtr, int ps, int cs,
                             bool rows_fast, int dir, const double2* __restrict__ tw, int nx) {
  const int L = 1 << lg;
  const int half = L >> 1;
  const int total = half << lgtr;
  for (int ns = 1; ns < L; ns <<= 1) {
    const int tws = nx / (2 * ns);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      int j, c;
      if (rows_fast) {
        j = idx & (half - 1);
        c = idx >> (lg - 1);
      } else {
        c = idx & ((1 << lgtr) - 1);
        j = idx >> lgtr;
      }
      const int k = j & (ns - 1);
      const double2 u = a[j * ps + c * cs];
      double2 v = a[(j + half) * ps + c * cs];
      double2 w = ld(&tw[k * tws]);
      if (dir > 0) w.y = -w.y;
      v = cmul(v, w);
      const int o = ((j - k) << 1) + k;
      b[o * ps + c * cs] = cadd(u, v);
      b[(o + ns) * ps + c * cs] = csub(u, v);
    }
    __syncthreads();
    double2* t = a;
    a = b;
    b = t;
  }
  return a;
}

__host__ __device__ inline int ilog2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

// Pass A: forward column FFTs (length n1) of field blockIdx.y, times the four-step twiddle.
__global__ void __launch_bounds__(kThreads) k_pstd_cols_fwd(int nx, int n1, int n2,
                                                            const double2* __restrict__ in0,
                                                            const double2* __restrict__ in1,
                                                            double2* __restrict__ Y,
                                                            const double2* __restrict__ tw) {
  extern __shared__ double2 sm[];
  double2* a = sm;
  double2* b = sm + n1 * kCols;
  const double2* x = blockIdx.y == 0 ? in0 : in1;
  const int c0 = blockIdx.x * kCols;
  for (int idx = threadIdx.x; idx < n1 * kCols; idx += blockDim.x) {
    const int c = idx & (kCols - 1), p = idx >> 3;
    a[p * kCols + c] = ld(&x[(long long)p * n2 + c0 + c]);
  }
  __syncthreads();
  const double2* r = smem_fft(a, b, ilog2(n1), 3, kCols, 1, false, -1, tw, nx);
  double2* y = Y + (long long)blockIdx.y * nx;
  for (int idx = threadIdx.x; idx < n1 * kCols; idx += blockDim.x) {
    const int c = idx & (kCols - 1), k1 = idx >> 3;
    y[(long long)k1 * n2 + c0 + c] = cmul(r[k1 * kCols + c], ld(&tw[(c0 + c) * k1]));
  }
}

// Pass B: rows k1 in [blockIdx.x kRows, +kRows).  kind 0: each field (blockIdx.y)
// times i q;  kind 1: (rho, Px) -> (-i rho - q Px) q / (eps (q^2 + small)) into
// field 0 (rhoPJ.py:836-866 restricted to x).
__global__ void __launch_bounds__(kThreads) k_pstd_rows(int nx, int n1, int n2, int kind,
                                                        double2* __restrict__ Y,
                                                        const double* __restrict__ q,
                                                        double small, double inv_eps,
                                                        const double2* __restrict__ tw) {
  extern __shared__ double2 sm[];
  const int nfl = kind == 1 ? 2 : 1;
  const int f0 = kind == 1 ? 0 : blockIdx.y;
  const int ntr = nfl * kRows;
  const int lg2 = ilog2(n2);
  double2* a = sm;
  double2* b = sm + ntr * n2;
  const int r0 = blockIdx.x * kRows;
  for (int idx = threadIdx.x; idx < ntr * n2; idx += blockDim.x) {
    const int t = idx >> lg2, p = idx & (n2 - 1);
    const int f = f0 + t / kRows, row = r0 + (t & (kRows - 1));
    a[t * n2 + p] = Y[(long long)f * nx + (long long)row * n2 + p];
  }
  __syncthreads();
  double2* r = smem_fft(a, b, lg2, ilog2(ntr), 1, n2, true, -1, tw, nx);
  for (int idx = threadIdx.x; idx < kRows * n2; idx += blockDim.x) {
    const int t = idx >> lg2, k2 = idx & (n2 - 1);
    const int k = r0 + t + n1 * k2;
    const double qk = q[k];
    if (kind == 0) {
      for (int g = 0; g < nfl; ++g) {
        const double2 v = r[(t + g * kRows) * n2 + k2];
        r[(t + g * kRows) * n2 + k2] = make_double2(-qk * v.y, qk * v.x);
      }
    } else {
      const double2 rho = r[t * n2 + k2];
      const double2 px = r[(t + kRows) * n2 + k2];
      const double qs = qk * qk + small;
      // rho_term = -i rho inv_eps / qs ; P_term = -(q Px) inv_eps / qs ; out = (rho_term + P_term) q
      const double2 rt = make_double2(rho.y * inv_eps / qs, -rho.x * inv_eps / qs);
      const double2 pt = make_double2(-(qk * px.x) * inv_eps / qs, -(qk * px.y) * inv_eps / qs);
      r[t * n2 + k2] = make_double2((rt.x + pt.x) * qk, (rt.y + pt.y) * qk);
    }
  }
  __syncthreads();
  const int ntr_out = kind == 1 ? kRows : ntr;
  double2* o = (r == a) ? b : a;
  const double2* s = smem_fft(r, o, lg2, ilog2(ntr_out), 1, n2, true, +1, tw, nx);
  for (int idx = threadIdx.x; idx < ntr_out * n2; idx += blockDim.x) {
    const int t = idx >> lg2, p = idx & (n2 - 1);
    const int f = f0 + t / kRows, k1 = r0 + (t & (kRows - 1));
    const double2 w = cconj(ld(&tw[p * k1]));
    Y[(long long)f * nx + (long long)k1 * n2 + p] = cmul(s[t * n2 + p], w);
  }
}

// Pass C: inverse column FFTs (length n1), 1/nx, epilogue.
__global__ void __launch_bounds__(kThreads) k_pstd_cols_inv(int nx, int n1, int n2,
                                                            const double2* __restrict__ Y,
                                                            const double2* __restrict__ tw,
                                                            const double* __restrict__ mask,
                                                            PstdEpiArgs e) {
  extern __shared__ double2 sm[];
  double2* a = sm;
  double2* b = sm + n1 * kCols;
  const int f = blockIdx.y;
  const double2* y = Y + (long long)f * nx;
  const int c0 = blockIdx.x * kCols;
  for (int idx = threadIdx.x; idx < n1 * kCols; idx += blockDim.x) {
    const int c = idx & (kCols - 1), k1 = idx >> 3;
    a[k1 * kCols + c] = y[(long long)k1 * n2 + c0 + c];
  }
  __syncthreads();
  const double2* r = smem_fft(a, b, ilog2(n1), 3, kCols, 1, false, +1, tw, nx);
  const double inv_n = 1.0 / (double)nx;
  double2* out = e.out[f];
  const double2* js = e.jsrc[f];
  for (int idx = threadIdx.x; idx < n1 * kCols; idx += blockDim.x) {
    const int c = idx & (kCols - 1), p = idx >> 3;
    const long long n = (long long)p * n2 + c0 + c;
    const double2 d = cscale(r[p * kCols + c], inv_n);
    if (e.mode == PSTD_STORE) {
      out[n] = d;
    } else {
      double2 v = out[n];
      v = make_double2(v.x + e.a[f] * d.x, v.y + e.a[f] * d.y);
      if (js) {
        const double2 j = js[n];
        v = make_double2(v.x + e.ja[f] * j.x, v.y + e.ja[f] * j.y);
      }
      if (e.masked) v = cscale(v, mask[n]);
      out[n] = v;
    }
  }
}

// Grid tables.  x follows numpy.linspace(-len/2, len/2, nx) (the driver's
// GetSpaceArray, PSTD3D/typespace.py:815-849): j * step + start, last = stop.
__global__ void k_pstd_tables(int nx, double dx, int n_abc, double strength, double2* tw,
                              double* q, double* x, double* mask) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nx) return;
  double s, c;
  sincospi(-2.0 * (double)j / (double)nx, &s, &c);
  tw[j] = make_double2(c, s);
  const double dq = 2.0 * kPi / ((double)nx * dx);  // helpers.py:854
  q[j] = (double)(j <= nx / 2 ? j : j - nx) * dq;
  const double len = (double)(nx - 1) * dx;
  const double start = -len / 2.0, stop = len / 2.0;
  const double step = (stop - start) / (double)(nx - 1);
  x[j] = (j == nx - 1) ? stop : __dadd_rn(__dmul_rn((double)j, step), start);
  const int d = min(j, nx - 1 - j);
  double m = 1.0;
  if (d < n_abc) {
    const double u = (double)(n_abc - d) / (double)n_abc;
    m = exp(-strength * u * u);
  }
  mask[j] = m;
}

bool g_attr_done[64] = {};

}  // namespace

int pstd_pipeline(SbePstd* p, int kind, const double2* in0, const double2* in1, int nf,
                  const PstdEpiArgs& epi, cudaStream_t s) {
  const int nx = p->nx, n1 = p->n1, n2 = p->n2;
  const size_t smA = 2 * (size_t)n1 * kCols * sizeof(double2);
  const size_t smB = 2 * (size_t)(kind == 1 ? 2 : 1) * kRows * n2 * sizeof(double2);
  k_pstd_cols_fwd<<<dim3(n2 / kCols, nf), kThreads, smA, s>>>(nx, n1, n2, in0, in1, p->work,
                                                              p->tw);
  // rhoPJ.py:779: small = (qx[1] - qx[0]) / 1e4, with q[0] = 0 and q[1] = dq
  const double dq = 2.0 * kPi / ((double)nx * p->dx);
  const double sm_q = dq / 1e4;
  const double inv_eps = 1.0 / (kEps0 * p->epsr);
  k_pstd_rows<<<dim3(n1 / kRows, kind == 1 ? 1 : nf), kThreads, smB, s>>>(
      nx, n1, n2, kind, p->work, p->q, sm_q, inv_eps, p->tw);
  const int nout = kind == 1 ? 1 : nf;
  k_pstd_cols_inv<<<dim3(n2 / kCols, nout), kThreads, smA, s>>>(nx, n1, n2, p->work, p->tw,
                                                               p->mask, epi);
  return cuda_check(cudaGetLastError(), "pstd pipeline");
}

}  // namespace sbe

using namespace sbe;

namespace {
int check_pstd(SbePstd* p, const char* who) {
  if (!p || !p->work) return fail(SBE_ERR_ARG, std::string(who) + ": null PSTD grid");
  return SBE_OK;
}
// Leapfrog stability of the spectral derivative: v dt q_max <= 2, q_max = pi / dx.
int check_dt(SbePstd* p, double dt, const char* who) {
  const double v = 299792458.0 / std::sqrt(p->epsr);
  if (!(dt > 0.0)) return fail(SBE_ERR_ARG, std::string(who) + ": dt must be > 0");
  if (v * dt * kPi / p->dx > 2.0)
    return fail(SBE_ERR_ARG, std::string(who) + ": unstable step, c dt pi / (sqrt(epsr) dx) = " +
                                 std::to_string(v * dt * kPi / p->dx) + " > 2");
  return SBE_OK;
}
}  // namespace

extern "C" {

int sbe_pstd_create(const SbePstdDesc* d, void* stream, SbePstd** out) {
  if (!d || !out) return fail(SBE_ERR_ARG, "sbe_pstd_create: null");
  *out = nullptr;
  const int nx = d->nx;
  if (nx < 256 || nx > 65536 || (nx & (nx - 1)))
    return fail(SBE_ERR_UNSUPPORTED, "sbe_pstd_create: nx must be a power of two in [256, 65536]");
  if (!(d->dx > 0.0) || !(d->epsr > 0.0) || d->n_abc < 0 || 2 * d->n_abc >= nx ||
      !(d->abc_strength >= 0.0))
    return fail(SBE_ERR_ARG, "sbe_pstd_create: bad dx / epsr / absorbing layer");
  SbePstd* p = new SbePstd();
  p->nx = nx;
  const int lg = ilog2(nx);
  p->n1 = 1 << (lg / 2);
  p->n2 = nx / p->n1;
  p->n_abc = d->n_abc;
  p->dx = d->dx;
  p->epsr = d->epsr;
  p->abc_strength = d->abc_strength;
  cudaGetDevice(&p->dev);
  cudaStream_t s = as_stream(stream);
  bool ok = cudaMalloc(&p->tw, sizeof(double2) * nx) == cudaSuccess &&
            cudaMalloc(&p->q, sizeof(double) * nx) == cudaSuccess &&
            cudaMalloc(&p->x, sizeof(double) * nx) == cudaSuccess &&
            cudaMalloc(&p->mask, sizeof(double) * nx) == cudaSuccess &&
            cudaMalloc(&p->work, sizeof(double2) * 2 * nx) == cudaSuccess;
  if (!ok) {
    sbe_pstd_destroy(p);
    return fail(SBE_ERR_OOM, "sbe_pstd_create: device allocation");
  }
  if (p->dev >= 0 && p->dev < 64 && !g_attr_done[p->dev]) {
    const int maxA = 2 * 256 * kCols * (int)sizeof(double2);
    const int maxB = 2 * 2 * kRows * 256 * (int)sizeof(double2);
    cudaFuncSetAttribute(k_pstd_cols_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, maxA);
    cudaFuncSetAttribute(k_pstd_cols_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, maxA);
    cudaFuncSetAttribute(k_pstd_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, maxB);
    g_attr_done[p->dev] = true;
  }
  k_pstd_tables<<<(nx + 255) / 256, 256, 0, s>>>(nx, d->dx, d->n_abc, d->abc_strength, p->tw,
                                                 p->q, p->x, p->mask);
  int rc = cuda_check(cudaGetLastError(), "sbe_pstd_create");
  if (rc == SBE_OK) rc = cuda_check(cudaStreamSynchronize(s), "sbe_pstd_create: tables");
  if (rc) {
    sbe_pstd_destroy(p);
    return rc;
  }
  *out = p;
  return SBE_OK;
}

int sbe_pstd_destroy(SbePstd* p) {
  if (!p) return SBE_OK;
  cudaFree(p->tw);
  cudaFree(p->q);
  cudaFree(p->x);
  cudaFree(p->mask);
  cudaFree(p->work);
  delete p;
  return SBE_OK;
}

int sbe_pstd_grid(SbePstd* p, double* x, double* q, void* stream) {
  int rc = check_pstd(p, "sbe_pstd_grid");
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);
  if (x) cudaMemcpyAsync(x, p->x, sizeof(double) * p->nx, cudaMemcpyDeviceToDevice, s);
  if (q) cudaMemcpyAsync(q, p->q, sizeof(double) * p->nx, cudaMemcpyDeviceToDevice, s);
  return cuda_check(cudaGetLastError(), "sbe_pstd_grid");
}

int sbe_pstd_deriv(SbePstd* p, const double* f, int nf, double* df, void* stream) {
  int rc = check_pstd(p, "sbe_pstd_deriv");
  if (rc) return rc;
  if (!f || !df || nf < 1 || nf > 2) return fail(SBE_ERR_ARG, "sbe_pstd_deriv: bad arguments");
  const double2* in = reinterpret_cast<const double2*>(f);
  double2* o = reinterpret_cast<double2*>(df);
  PstdEpiArgs e;
  e.mode = PSTD_STORE;
  e.out[0] = o;
  e.out[1] = o + p->nx;
  return pstd_pipeline(p, 0, in, in + p->nx, nf, e, as_stream(stream));
}

int sbe_pstd_update_h(SbePstd* p, const double* E, double* H, double dt, void* stream) {
  int rc = check_pstd(p, "sbe_pstd_update_h");
  if (rc) return rc;
  if (!E || !H) return fail(SBE_ERR_ARG, "sbe_pstd_update_h: null field");
  if ((rc = check_dt(p, dt, "sbe_pstd_update_h"))) return rc;
  const double2* e2 = reinterpret_cast<const double2*>(E);
  double2* h2 = reinterpret_cast<double2*>(H);
  PstdEpiArgs e;
  e.mode = PSTD_UPDATE;
  e.out[0] = h2;           // Hz -= dt/mu0 d_x Ey
  e.out[1] = h2 + p->nx;   // Hy += dt/mu0 d_x Ez
  e.a[0] = -dt / kMu0;
  e.a[1] = dt / kMu0;
  e.masked = p->n_abc > 0;
  return pstd_pipeline(p, 0, e2, e2 + p->nx, 2, e, as_stream(stream));
}

int sbe_pstd_update_e(SbePstd* p, double* E, const double* H, const double* J, double dt,
                      void* stream) {
  int rc = check_pstd(p, "sbe_pstd_update_e");
  if (rc) return rc;
  if (!E || !H) return fail(SBE_ERR_ARG, "sbe_pstd_update_e: null field");
  if ((rc = check_dt(p, dt, "sbe_pstd_update_e"))) return rc;
  double2* e2 = reinterpret_cast<double2*>(E);
  const double2* h2 = reinterpret_cast<const double2*>(H);
  const double2* j2 = reinterpret_cast<const double2*>(J);
  const double ie = dt / (kEps0 * p->epsr);
  PstdEpiArgs e;
  e.mode = PSTD_UPDATE;
  e.out[0] = e2;           // Ey -= dt/eps (d_x Hz + Jy)
  e.out[1] = e2 + p->nx;   // Ez += dt/eps (d_x Hy - Jz)
  e.a[0] = -ie;
  e.a[1] = ie;
  if (j2) {
    e.jsrc[0] = j2;
    e.jsrc[1] = j2 + p->nx;
    e.ja[0] = -ie;
    e.ja[1] = -ie;
  }
  e.masked = p->n_abc > 0;
  return pstd_pipeline(p, 0, h2, h2 + p->nx, 2, e, as_stream(stream));
}

int sbe_pstd_step(SbePstd* p, double* E, double* H, const double* J, double dt, void* stream) {
  int rc = sbe_pstd_update_h(p, E, H, dt, stream);
  if (rc) return rc;
  return sbe_pstd_update_e(p, E, H, J, dt, stream);
}

int sbe_pstd_elong(SbePstd* p, const double* rho, const double* Px, double* Ex, void* stream) {
  int rc = check_pstd(p, "sbe_pstd_elong");
  if (rc) return rc;
  if (!rho || !Px || !Ex) return fail(SBE_ERR_ARG, "sbe_pstd_elong: null");
  PstdEpiArgs e;
  e.mode = PSTD_STORE;
  e.out[0] = reinterpret_cast<double2*>(Ex);
  return pstd_pipeline(p, 1, reinterpret_cast<const double2*>(rho),
                       reinterpret_cast<const double2*>(Px), 2, e, as_stream(stream));
}

}  // extern "C"
