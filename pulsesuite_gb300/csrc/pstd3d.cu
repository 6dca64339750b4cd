// 3-D PSTD field step: six field components on an nx x ny x nz grid (C order, z
// fastest), spectral curls by 3-D FFTs built from three axis passes, the k-space
// curl multiply fused into the x pass and the field update fused into the last
// (inverse z) pass.
//
// The reference has no 3-D Maxwell stepper either (its 3-D driver sets E
// analytically, sbetestpropnov30.py:709); the pieces are the q-space derivative
// f (i q) along each axis (PSTD3D/usefulsubs.py:233-380), the grids of
// typespace.py:815-849 and helpers.py:838-863, the absorbing mask multiply of
// ApplyABC (usefulsubs.py:584-609) and the longitudinal field of ElongfromRho
// (rhoPJ.py:703-880).  Leapfrog:
//   H^{n+1/2} = H^{n-1/2} - dt/mu0 curl E^n,
//   E^{n+1}   = mask (E^n + dt/eps (curl H^{n+1/2} - J)).
//
// One curl of a field triple F (3 x c128 N, N = nx ny nz) runs five passes:
//   1  z lines, forward (FP64 field -> work W)
//   2  y lines, forward (in place)
//   3  x lines: forward, c = i q x F at every (kx, ky, kz), inverse (in place; a block
//      holds the x lines of all three components of its (ky, kz) columns)
//   4  y lines, inverse
//   5  z lines, inverse, 1/N, and out += a c (+ ja J), mask (FP64 out)
// Every transform is a radix-2 Stockham sequence in shared memory.  The work array
// W is FP64 or FP32 complex (chosen at creation): with FP32 work the three middle
// passes move half the bytes and the FP64 field is touched only by passes 1 and 5.
#include <cmath>
#include <vector>

#include "fp_bits.cuh"
#include "pstd3d.cuh"

namespace sbe {
namespace {

constexpr double kMu0 = 1.25663706127e-6;   // CODATA 2022 (scipy.constants.mu_0)
constexpr int kThreads = 256;
constexpr int kSmemMax = 200 * 1024;

template <typename T>
__device__ __forceinline__ T mk(double a, double b);
template <>
__device__ __forceinline__ double2 mk<double2>(double a, double b) {
  return make_double2(a, b);
}
template <>
__device__ __forceinline__ float2 mk<float2>(double a, double b) {
  return make_float2((float)a, (float)b);
}

template <typename T>
__device__ __forceinline__ T tmul(T a, T b) {
  T r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

template <typename T>
__device__ __forceinline__ T twd(const double2* tw, const float2* twf, int i);
template <>
__device__ __forceinline__ double2 twd<double2>(const double2* tw, const float2*, int i) {
  return __ldg(&tw[i]);
}
template <>
__device__ __forceinline__ float2 twd<float2>(const double2*, const float2* twf, int i) {
  return __ldg(&twf[i]);
}

// Radix-2 Stockham over shared memory: ntr = 2^lgtr transforms of length L = 2^lg,
// element p of transform c at a[p * ps + c * cs]; consecutive threads walk c
// (c_fast) or p.  dir -1: exp(-i ...), +1: exp(+i ...).  Returns the buffer
// holding the result in natural order.
template <typename T>
__device__ T* fft_smem(T* a, T* b, int lg, int lgtr, int ps, int cs, bool c_fast, int dir,
                       const double2* tw, const float2* twf) {
  const int L = 1 << lg;
  const int half = L >> 1;
  const int total = half << lgtr;
  for (int ns = 1; ns < L; ns <<= 1) {
    const int tws = L / (2 * ns);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      int j, c;
      if (c_fast) {
        c = idx & ((1 << lgtr) - 1);
        j = idx >> lgtr;
      } else {
        j = idx & (half - 1);
        c = idx >> (lg - 1);
      }
      const int k = j & (ns - 1);
      const T u = a[j * ps + c * cs];
      T v = a[(j + half) * ps + c * cs];
      T w = twd<T>(tw, twf, k * tws);
      if (dir > 0) w.y = -w.y;
      v = tmul(v, w);
      const int o = ((j - k) << 1) + k;
      T s0, s1;
      s0.x = u.x + v.x;
      s0.y = u.y + v.y;
      s1.x = u.x - v.x;
      s1.y = u.y - v.y;
      b[o * ps + c * cs] = s0;
      b[(o + ns) * ps + c * cs] = s1;
    }
    __syncthreads();
    T* t = a;
    a = b;
    b = t;
  }
  return a;
}

__host__ __device__ inline int ilog2i(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

// Geometry of one pass: lines of length n along an axis of stride s (elements);
// lines are enumerated by (outer o, inner i), element p of line (o, i) at
// o * n * s + p * s + i (field f at f * N).
struct Pass {
  int n, lg, s, inner, tl, lgtl, nf;
  long long N;
  int dir;
  const double2* tw;
  const float2* twf;
};

// Generic line pass: nf fields.  Loads TL lines of each field (consecutive inner
// indices, or consecutive whole lines when s == 1), transforms them, stores them.
// in64 / out64: FP64 fields (pass 1 reads one, pass 5 writes one through the update
// epilogue); otherwise the work array (T) is read and written in place.
struct Upd {
  double2* out;            // FP64 destination (nullptr: store to work)
  const double2* J;        // optional current (FP64, 3 fields)
  double a, ja;            // out += a * result / N - ja * J
  const double* m0;        // masks per axis (nullptr: none)
  const double* m1;
  const double* m2;
  int nx, ny, nz;
  int store;               // 1: out = result / N (no update)
  float af[2], jf[2];      // the plane path's a / N and ja as FP32 pairs (hi, lo)
  int nabc[3];             // absorbing widths: the mask is exactly 1 further inside
};

template <typename T>
__global__ void __launch_bounds__(kThreads) k_line_pass(Pass P, const double2* in64, T* W,
                                                        Upd U) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sa = reinterpret_cast<T*>(smraw);
  const int tl = P.tl, n = P.n;
  const int f = blockIdx.y;   // field
  T* sb = sa + (size_t)n * tl;
  // line block: lines (o, i0 .. i0 + tl - 1), or tl whole lines when s == 1
  long long base;
  if (P.s == 1) {
    base = (long long)blockIdx.x * tl * n;    // lines contiguous, element (c, p) at c n + p
  } else {
    const int bpo = P.inner / tl;             // blocks per outer index
    const int o = blockIdx.x / bpo, i0 = (blockIdx.x % bpo) * tl;
    base = (long long)o * n * P.s + i0;
  }
  const long long fo = (long long)f * P.N;
  const int total = n * tl;
  // smem layout: element p of line c at p * tl + c (strided) or c * n + p (s == 1)
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    long long g;
    int sm;
    if (P.s == 1) {
      g = base + idx;                          // c = idx / n, p = idx % n
      sm = idx;
    } else {
      const int c = idx % tl, p = idx / tl;
      g = base + (long long)p * P.s + c;
      sm = p * tl + c;
    }
    T v;
    if (in64) {
      const double2 d = in64[fo + g];
      v = mk<T>(d.x, d.y);
    } else {
      v = W[fo + g];
    }
    sa[sm] = v;
  }
  __syncthreads();
  T* r;
  if (P.s == 1)
    r = fft_smem(sa, sb, P.lg, P.lgtl, 1, n, false, P.dir, P.tw, P.twf);
  else
    r = fft_smem(sa, sb, P.lg, P.lgtl, tl, 1, true, P.dir, P.tw, P.twf);
  const double invN = 1.0 / (double)((long long)U.nx * U.ny * U.nz);
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    long long g;
    int sm;
    if (P.s == 1) {
      g = base + idx;
      sm = idx;
    } else {
      const int c = idx % tl, p = idx / tl;
      g = base + (long long)p * P.s + c;
      sm = p * tl + c;
    }
    const T v = r[sm];
    if (!U.out) {
      W[fo + g] = v;
      continue;
    }
    double vx = (double)v.x * invN, vy = (double)v.y * invN;
    double2 o;
    if (U.store) {
      o = make_double2(vx, vy);
    } else {
      o = U.out[fo + g];
      o.x += U.a * vx;
      o.y += U.a * vy;
      if (U.J) {
        const double2 j = U.J[fo + g];
        o.x -= U.ja * j.x;
        o.y -= U.ja * j.y;
      }
    }
    if (U.m0) {
      const long long yz = (long long)U.ny * U.nz;
      const int i = (int)(g / yz), jj = (int)((g / U.nz) % U.ny), k = (int)(g % U.nz);
      const double m = U.m0[i] * U.m1[jj] * U.m2[k];
      o.x *= m;
      o.y *= m;
    }
    U.out[fo + g] = o;
  }
}

// The x pass of the curl: a block holds the x lines of the three components of tl
// consecutive (y, z) columns; forward FFT, c = i q x F, inverse FFT, in place.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_x_curl(Pass P, T* W, const double* qy,
                                                     const double* qz, const double* qx, int nz) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sa = reinterpret_cast<T*>(smraw);
  const int tl = P.tl, n = P.n;
  T* sb = sa + (size_t)3 * n * tl;
  const int b0 = blockIdx.x * tl;             // first (y, z) column
  const int total = 3 * n * tl;               // element (f, p, c) at (f * n + p) * tl + c
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int c = idx % tl, fp = idx / tl, p = fp % n, f = fp / n;
    sa[idx] = W[(long long)f * P.N + (long long)p * P.s + b0 + c];
  }
  __syncthreads();
  // 3 tl transforms: transform index t = f * tl + c, element p at (f n + p) tl + c =
  // p tl + (f n tl + c): not a single stride, so transform each component in turn
  T* r[3];
  for (int f = 0; f < 3; ++f)
    r[f] = fft_smem(sa + (size_t)f * n * tl, sb + (size_t)f * n * tl, P.lg, P.lgtl, tl, 1, true,
                    -1, P.tw, P.twf);
  // the curl at every (kx, column)
  for (int idx = threadIdx.x; idx < n * tl; idx += blockDim.x) {
    const int c = idx % tl, p = idx / tl;
    const int col = b0 + c;
    const double kx = qx[p], ky = qy[col / nz], kz = qz[col % nz];
    const T fx = r[0][idx], fy = r[1][idx], fz = r[2][idx];
    // i (k x F)
    const double cxr = ky * fz.x - kz * fy.x, cxi = ky * fz.y - kz * fy.y;
    const double cyr = kz * fx.x - kx * fz.x, cyi = kz * fx.y - kx * fz.y;
    const double czr = kx * fy.x - ky * fx.x, czi = kx * fy.y - ky * fx.y;
    r[0][idx] = mk<T>(-cxi, cxr);
    r[1][idx] = mk<T>(-cyi, cyr);
    r[2][idx] = mk<T>(-czi, czr);
  }
  __syncthreads();
  T* o[3];
  for (int f = 0; f < 3; ++f) {
    T* other = (r[f] == sa + (size_t)f * n * tl) ? sb + (size_t)f * n * tl : sa + (size_t)f * n * tl;
    o[f] = fft_smem(r[f], other, P.lg, P.lgtl, tl, 1, true, +1, P.tw, P.twf);
  }
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int c = idx % tl, fp = idx / tl, p = fp % n, f = fp / n;
    W[(long long)f * P.N + (long long)p * P.s + b0 + c] = o[f][p * tl + c];
  }
}

// ElongfromRho in k space (rhoPJ.py:836-866) on the transformed fields
// S = [rho, Px, Py, Pz]: writes the ten spectra [E_PRho x, y, z, E_P x, y, z,
// E_Rho x, y, z, rho_B] into O.  small = (qx[1] - qx[0]) / 1e4 (:779).
__global__ void k_elong3(long long N, int ny, int nz, const double2* S, double2* O,
                         const double* qx, const double* qy, const double* qz, double small,
                         double inv_eps) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= N) return;
  const long long yz = (long long)ny * nz;
  const double kx = qx[g / yz], ky = qy[(g / nz) % ny], kz = qz[g % nz];
  const double2 rk = S[g], px = S[N + g], py = S[2 * N + g], pz = S[3 * N + g];
  const double qs = kx * kx + ky * ky + kz * kz + small;
  const double2 qp = make_double2(kx * px.x + ky * py.x + kz * pz.x, kx * px.y + ky * py.y + kz * pz.y);
  // rho_term = -i rho inv_eps / qs ; P_term = -(q.P) inv_eps / qs
  const double2 rt = make_double2(rk.y * inv_eps / qs, -rk.x * inv_eps / qs);
  const double2 pt = make_double2(-qp.x * inv_eps / qs, -qp.y * inv_eps / qs);
  const double q3[3] = {kx, ky, kz};
  for (int c = 0; c < 3; ++c) {
    O[(long long)c * N + g] = make_double2((rt.x + pt.x) * q3[c], (rt.y + pt.y) * q3[c]);
    O[(long long)(3 + c) * N + g] = make_double2(pt.x * q3[c], pt.y * q3[c]);
    O[(long long)(6 + c) * N + g] = make_double2(rt.x * q3[c], rt.y * q3[c]);
  }
  O[9 * N + g] = make_double2(qp.y, -qp.x);   // rho_B = -i q.P
}

__global__ void k_tables3(int n, double d, double* x, double* q, double2* tw, float2* twf,
                          float2* qb, double* mask, int n_abc, double strength) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  {
    // the wavenumber of bit-reversed position j as an FP32 pair (the plane path's
    // spectrum order)
    int lg = 0;
    while ((1 << lg) < n) ++lg;
    const int jb = (int)(__brev((unsigned)j) >> (32 - lg));
    const double qv = (jb <= n / 2 ? jb : jb - n) * (2.0 * kPi / (n * d));
    const float hi = (float)qv;
    qb[j] = make_float2(hi, (float)(qv - (double)hi));
  }
  // GetSpaceArray: numpy linspace(-L/2, L/2, n) with L = (n - 1) d (typespace.py:815-849):
  // j * step + start, rounded as numpy does (no fused multiply-add), the last point = stop
  const double L = (n - 1) * d;
  const double start = -L / 2, stop = L / 2;
  const double step = (stop - start) / (double)(n - 1);
  x[j] = (j == n - 1) ? stop : __dadd_rn(__dmul_rn((double)j, step), start);
  const double dq = 2.0 * kPi / (n * d);
  q[j] = (j <= n / 2 ? j : j - n) * dq;
  double s, c;
  sincospi(-2.0 * (double)j / (double)n, &s, &c);
  tw[j] = make_double2(c, s);
  twf[j] = make_float2((float)c, (float)s);
  const int dd = j < n - 1 - j ? j : n - 1 - j;
  double m = 1.0;
  if (n_abc > 0 && dd < n_abc) {
    const double u = (double)(n_abc - dd) / n_abc;
    m = exp(-strength * u * u);
  }
  mask[j] = m;
}

// ---- FP32 work with (y, z) planes in shared memory: three passes per curl ------
// When a (y, z) plane of FP32 complex values fits in one block's shared memory
// (ny nz <= kPlaneMax) a curl is three passes instead of five:
//   A  per (x, component) plane: FP64 field -> FP32, forward transforms along z and y
//   B  x lines of tl (y, z) columns of all three components: forward along x, the curl
//      i q x F, inverse along x
//   C  per plane: inverse along y and z, out (+)= a curl / N (- ja J), mask; in the
//      field step C of the H update continues with pass A of the E update on the new
//      H it has just written (the plane is still in shared memory)
// The transforms run in place: radix-2 decimation in frequency (natural order in,
// bit-reversed order out, exp(-i ...)) and its exact inverse, decimation in time
// (bit-reversed in, natural out, unnormalised), two radix-2 stages fused per sweep
// over shared memory.  The spectrum is never reordered: the curl is pointwise in k
// space and reads the wavenumber of position p as q[bitrev(p)].
constexpr int kPlaneMax = 16384;   // FP32 complex elements of one plane (128 KB)
constexpr int kPlaneThreads = 1024;
constexpr int kXThreads = 512;
constexpr int kXSmem = 96 * 1024;  // shared memory of one x-pass block's lines

__device__ __forceinline__ float2 c_mul(float2 a, float2 w) {
  return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
__device__ __forceinline__ float2 c_mulc(float2 a, float2 w) {   // a conj(w)
  return make_float2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ int brev(int p, int lg) { return lg ? (int)(__brev((unsigned)p) >> (32 - lg)) : 0; }

// nl lines of n = 2^lg elements in shared memory, element p of line l at logical
// index i = l * ls + p * es, stored at a[i + (i >> psh)] (psh > 0: one padding slot
// after every 2^psh elements; the planes pad each row of nz, so that rows start on
// successive banks); tw[j] = exp(-2 pi i j / n), j < n / 2.  line_fast: consecutive
// threads take consecutive lines, else consecutive positions of one line.  Ends with
// __syncthreads.
__device__ __forceinline__ int smi(int i, int psh) { return psh ? i + (i >> psh) : i; }

template <bool INV>
__device__ void fft_inplace(float2* a, int lg, int nl, int ls, int es, bool line_fast,
                            const float2* tw, int psh) {
  const int n = 1 << lg, npair = lg >> 1, q4 = n >> 2;
  if ((lg & 1) && INV) {
    // the radix-2 stage of span 1 (twiddle 1): first for DIT, last for DIF
    for (int u = threadIdx.x; u < nl * (n >> 1); u += blockDim.x) {
      const int l = line_fast ? u % nl : u / (n >> 1), b = line_fast ? u / nl : u % (n >> 1);
      const int i0 = l * ls + 2 * b * es;
      const float2 x0 = a[smi(i0, psh)], x1 = a[smi(i0 + es, psh)];
      a[smi(i0, psh)] = c_add(x0, x1);
      a[smi(i0 + es, psh)] = c_sub(x0, x1);
    }
    __syncthreads();
  }
  for (int t = 0; t < npair; ++t) {
    const int pi = INV ? npair - 1 - t : t;
    const int m = n >> (2 * pi + 2), lgm = lg - 2 * pi - 2;
    const int tws = q4 / m;     // n / (4 m): w_{4m}^j = tw[j tws]
    for (int u = threadIdx.x; u < nl * q4; u += blockDim.x) {
      const int l = line_fast ? u % nl : u / q4, r = line_fast ? u / nl : u % q4;
      const int j = r & (m - 1), p0 = ((r >> lgm) << (lgm + 2)) + j;
      const int sm = m * es, i0 = l * ls + p0 * es;
      const int k0 = smi(i0, psh), k1 = smi(i0 + sm, psh), k2 = smi(i0 + 2 * sm, psh),
                k3 = smi(i0 + 3 * sm, psh);
      const float2 x0 = a[k0], x1 = a[k1], x2 = a[k2], x3 = a[k3];
      const float2 w1a = tw[j * tws], w1b = tw[(j + m) * tws], w2 = tw[2 * j * tws];
      float2 y0, y1, y2, y3;
      if (!INV) {
        const float2 a0 = c_add(x0, x2), a2 = c_mul(c_sub(x0, x2), w1a);
        const float2 a1 = c_add(x1, x3), a3 = c_mul(c_sub(x1, x3), w1b);
        y0 = c_add(a0, a1);
        y1 = c_mul(c_sub(a0, a1), w2);
        y2 = c_add(a2, a3);
        y3 = c_mul(c_sub(a2, a3), w2);
      } else {
        const float2 t1 = c_mulc(x1, w2), t3 = c_mulc(x3, w2);
        const float2 a0 = c_add(x0, t1), a1 = c_sub(x0, t1);
        const float2 a2 = c_add(x2, t3), a3 = c_sub(x2, t3);
        const float2 t2 = c_mulc(a2, w1a), t4 = c_mulc(a3, w1b);
        y0 = c_add(a0, t2);
        y2 = c_sub(a0, t2);
        y1 = c_add(a1, t4);
        y3 = c_sub(a1, t4);
      }
      a[k0] = y0;
      a[k1] = y1;
      a[k2] = y2;
      a[k3] = y3;
    }
    __syncthreads();
  }
  if ((lg & 1) && !INV) {
    for (int u = threadIdx.x; u < nl * (n >> 1); u += blockDim.x) {
      const int l = line_fast ? u % nl : u / (n >> 1), b = line_fast ? u / nl : u % (n >> 1);
      const int i0 = l * ls + 2 * b * es;
      const float2 x0 = a[smi(i0, psh)], x1 = a[smi(i0 + es, psh)];
      a[smi(i0, psh)] = c_add(x0, x1);
      a[smi(i0 + es, psh)] = c_sub(x0, x1);
    }
    __syncthreads();
  }
}

struct PlaneArgs {
  int lgy, lgz, ny, nz, nx;
  long long N, P;                 // grid points, points per (y, z) plane
  const float2* twy;              // exp(-2 pi i j / ny), j < ny (global)
  const float2* twz;
};

// padded plane of P elements in shared memory
__host__ __device__ inline long long plane_slots(long long P, int lgz) { return P + (P >> lgz); }

// shared memory of a plane block: the padded plane, then the y and z twiddles (half each)
__device__ __forceinline__ void plane_tables(const PlaneArgs& A, float2* sty, float2* stz) {
  for (int j = threadIdx.x; j < (A.ny >> 1); j += blockDim.x) sty[j] = A.twy[j];
  for (int j = threadIdx.x; j < (A.nz >> 1); j += blockDim.x) stz[j] = A.twz[j];
}

// forward along z (rows of the plane) then y (columns)
__device__ __forceinline__ void plane_forward(const PlaneArgs& A, float2* a, const float2* sty,
                                              const float2* stz) {
  // both directions with consecutive threads on consecutive lines: along z the lines
  // are the padded rows (successive banks), along y the adjacent columns
  fft_inplace<false>(a, A.lgz, A.ny, A.nz, 1, true, stz, A.lgz);
  fft_inplace<false>(a, A.lgy, A.nz, 1, A.nz, true, sty, A.lgz);
}

// pass A: plane (x = blockIdx.x, component blockIdx.y) of the FP64 field F -> W
// (FP64 -> FP32 on the integer pipe: the FP64 pipe is ~1/64 of the FP32 rate here)
__global__ void __launch_bounds__(kPlaneThreads, 1) k_plane_fwd(PlaneArgs A, const double2* F,
                                                                float2* W) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* a = reinterpret_cast<float2*>(smraw);
  float2* sty = a + plane_slots(A.P, A.lgz);
  float2* stz = sty + (A.ny >> 1);
  const long long base = blockIdx.y * A.N + blockIdx.x * A.P;
  plane_tables(A, sty, stz);
  // all loads of a thread before the stores to shared memory (4 per round)
  for (int i0 = threadIdx.x; i0 < A.P; i0 += 4 * kPlaneThreads) {
    double2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * kPlaneThreads;
      v[u] = i < A.P ? F[base + i] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * kPlaneThreads;
      if (i < A.P) a[smi(i, A.lgz)] = f64_to_f32(v[u]);
    }
  }
  __syncthreads();
  plane_forward(A, a, sty, stz);
  for (int i = threadIdx.x; i < A.P; i += kPlaneThreads) W[base + i] = a[smi(i, A.lgz)];
}

// pass B: the x lines of tl consecutive (y, z) columns of all three components;
// shared memory [x][component][column].  qb*: the wavenumbers of the bit-reversed
// positions as FP32 pairs (hi, lo): k f = fmaf(hi, f, lo f), one rounding per
// product (an FP32 wavenumber alone is up to 6e-8 off, a fixed phase-velocity error
// of its mode)
__global__ void __launch_bounds__(kXThreads) k_x_curl_ip(PlaneArgs A, float2* W, int lgx, int tl,
                                                         const float2* twx, const float2* qbx,
                                                         const float2* qby, const float2* qbz) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = 1 << lgx, w3 = 3 * tl;
  float2* a = reinterpret_cast<float2*>(smraw);
  float2* stx = a + (size_t)nx * w3;
  for (int j = threadIdx.x; j < (nx >> 1); j += blockDim.x) stx[j] = twx[j];
  const long long b0 = (long long)blockIdx.x * tl;
  const int total = nx * w3;
  // four loads of a thread in flight before their stores to shared memory
  for (int i0 = threadIdx.x; i0 < total; i0 += 4 * kXThreads) {
    float2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int idx = i0 + u * kXThreads;
      if (idx < total) {
        const int px = idx / w3, r = idx - px * w3, f = r / tl, c = r - f * tl;
        v[u] = W[f * A.N + px * A.P + b0 + c];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (i0 + u * kXThreads < total) a[i0 + u * kXThreads] = v[u];
  }
  __syncthreads();
  fft_inplace<false>(a, lgx, w3, 1, w3, true, stx, 0);
  for (int idx = threadIdx.x; idx < nx * tl; idx += blockDim.x) {
    const int px = idx / tl, c = idx - px * tl;
    const long long col = b0 + c;
    const int py = (int)(col >> A.lgz), pz = (int)(col & (A.nz - 1));
    const float2 kx = qbx[px], ky = qby[py], kz = qbz[pz];
    float2* e = a + (size_t)px * w3 + c;
    const float2 fx = e[0], fy = e[tl], fz = e[2 * tl];
    auto km = [](float2 k, float f) { return fmaf(k.x, f, k.y * f); };
    // i (k x F)
    const float cxr = km(ky, fz.x) - km(kz, fy.x), cxi = km(ky, fz.y) - km(kz, fy.y);
    const float cyr = km(kz, fx.x) - km(kx, fz.x), cyi = km(kz, fx.y) - km(kx, fz.y);
    const float czr = km(kx, fy.x) - km(ky, fx.x), czi = km(kx, fy.y) - km(ky, fx.y);
    e[0] = make_float2(-cxi, cxr);
    e[tl] = make_float2(-cyi, cyr);
    e[2 * tl] = make_float2(-czi, czr);
  }
  __syncthreads();
  fft_inplace<true>(a, lgx, w3, 1, w3, true, stx, 0);
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int px = idx / w3, r = idx - px * w3, f = r / tl, c = r - f * tl;
    W[f * A.N + px * A.P + b0 + c] = a[idx];
  }
}

// pass C: inverse along y and z of plane (x, component), then out (+)= ...: the
// update of Upd (the masks per axis); with fwd_next the plane of the updated FP64
// field continues as pass A of the next curl (W overwritten with its transform: the
// block owns its plane of W).  The increment a v / N - ja J is formed in FP32 (v is
// the FP32 transform; a / N and ja as FP32 pairs, J rounded to FP32 on the integer
// pipe) and added to the FP64 field: one FP64 add per component; the mask multiplies
// only where it is not 1.
__global__ void __launch_bounds__(kPlaneThreads, 1) k_plane_inv(PlaneArgs A, float2* W, Upd U,
                                                                int fwd_next) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* a = reinterpret_cast<float2*>(smraw);
  float2* sty = a + plane_slots(A.P, A.lgz);
  float2* stz = sty + (A.ny >> 1);
  const int x = blockIdx.x;
  const long long base = blockIdx.y * A.N + x * A.P;
  plane_tables(A, sty, stz);
  for (int i = threadIdx.x; i < A.P; i += kPlaneThreads) a[smi(i, A.lgz)] = W[base + i];
  __syncthreads();
  fft_inplace<true>(a, A.lgy, A.nz, 1, A.nz, true, sty, A.lgz);
  fft_inplace<true>(a, A.lgz, A.ny, A.nz, 1, true, stz, A.lgz);
  const double mx = U.m0 ? U.m0[x] : 1.0;
  const bool xin = min(x, A.nx - 1 - x) >= U.nabc[0];
  for (int i0 = threadIdx.x; i0 < A.P; i0 += 2 * kPlaneThreads) {
    // both elements' FP64 loads before their updates
    double2 o[2], jv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int i = i0 + u * kPlaneThreads;
      const bool in = i < A.P;
      o[u] = (in && !U.store) ? U.out[base + i] : make_double2(0.0, 0.0);
      jv[u] = (in && U.J) ? U.J[base + i] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int i = i0 + u * kPlaneThreads;
      if (i >= A.P) continue;
      const float2 v = a[smi(i, A.lgz)];
      float ix = fmaf(v.x, U.af[0], v.x * U.af[1]), iy = fmaf(v.y, U.af[0], v.y * U.af[1]);
      if (U.J) {
        const float2 jf = f64_to_f32(jv[u]);
        ix -= fmaf(jf.x, U.jf[0], jf.x * U.jf[1]);
        iy -= fmaf(jf.y, U.jf[0], jf.y * U.jf[1]);
      }
      double2 r = make_double2(o[u].x + f32_to_f64(ix), o[u].y + f32_to_f64(iy));
      if (U.m0) {
        // FP64 only inside the absorbing layers (integer test of the position)
        const int y = i >> A.lgz, z = i & (A.nz - 1);
        if (!xin || min(y, A.ny - 1 - y) < U.nabc[1] || min(z, A.nz - 1 - z) < U.nabc[2]) {
          const double m = mx * U.m1[y] * U.m2[z];
          r.x *= m;
          r.y *= m;
        }
      }
      U.out[base + i] = r;
      if (fwd_next) a[smi(i, A.lgz)] = f64_to_f32(r);
    }
  }
  if (!fwd_next) return;   // block-uniform
  __syncthreads();
  plane_forward(A, a, sty, stz);
  for (int i = threadIdx.x; i < A.P; i += kPlaneThreads) W[base + i] = a[smi(i, A.lgz)];
}

bool pow2(int v) { return v >= 2 && v <= 1024 && (v & (v - 1)) == 0; }

// tl lines per block within the shared-memory budget (two ping-pong buffers of nf
// fields x n x tl elements), tl <= 8 and dividing inner
int lines_per_block(int n, int nf, size_t elem, int inner) {
  int tl = 8;
  while (tl > 1 && (2 * (size_t)nf * n * tl * elem > (size_t)kSmemMax || inner % tl)) tl >>= 1;
  return tl;
}

template <typename T>
int run_line_pass(SbePstd3* p, int axis, int dir, int nf, const double2* in64, T* W,
                  const Upd& U, cudaStream_t s) {
  Pass P{};
  P.n = p->n[axis];
  P.lg = ilog2i(P.n);
  P.s = axis == 2 ? 1 : (axis == 1 ? p->n[2] : p->n[1] * p->n[2]);
  P.inner = P.s;
  P.N = p->N;
  P.nf = nf;
  P.dir = dir;
  P.tw = p->tw[axis];
  P.twf = p->twf[axis];
  const int lines = (int)(p->N / P.n);
  P.tl = P.s == 1 ? 8 : lines_per_block(P.n, 1, sizeof(T), P.inner);
  if (P.s == 1)
    while (P.tl > 1 && 2 * (size_t)P.n * P.tl * sizeof(T) > (size_t)kSmemMax) P.tl >>= 1;
  P.lgtl = ilog2i(P.tl);
  const size_t smem = 2 * (size_t)P.n * P.tl * sizeof(T);
  const dim3 grid(lines / P.tl, nf);
  k_line_pass<T><<<grid, kThreads, smem, s>>>(P, in64, W, U);
  return cuda_check(cudaGetLastError(), "pstd3 line pass");
}

template <typename T>
int run_x_curl(SbePstd3* p, T* W, cudaStream_t s) {
  Pass P{};
  P.n = p->n[0];
  P.lg = ilog2i(P.n);
  P.s = p->n[1] * p->n[2];
  P.inner = P.s;
  P.N = p->N;
  P.tw = p->tw[0];
  P.twf = p->twf[0];
  P.tl = lines_per_block(P.n, 3, sizeof(T), P.inner);
  P.lgtl = ilog2i(P.tl);
  const size_t smem = 2 * 3 * (size_t)P.n * P.tl * sizeof(T);
  k_x_curl<T><<<P.s / P.tl, kThreads, smem, s>>>(P, W, p->q[1], p->q[2], p->q[0], p->n[2]);
  return cuda_check(cudaGetLastError(), "pstd3 curl pass");
}

Upd upd_store(SbePstd3* p) {
  Upd U{};
  U.nx = p->n[0];
  U.ny = p->n[1];
  U.nz = p->n[2];
  return U;
}

// out (+)= curl F: a, ja, J, masked as in Upd (store = 1: out = curl F).
template <typename T>
int curl_pipeline(SbePstd3* p, const double2* F, double2* out, double a, const double2* J,
                  double ja, bool masked, int store, cudaStream_t s) {
  T* W = static_cast<T*>(p->work);
  Upd none = upd_store(p);
  int rc = run_line_pass<T>(p, 2, -1, 3, F, W, none, s);
  if (!rc) rc = run_line_pass<T>(p, 1, -1, 3, nullptr, W, none, s);
  if (!rc) rc = run_x_curl<T>(p, W, s);
  if (!rc) rc = run_line_pass<T>(p, 1, +1, 3, nullptr, W, none, s);
  if (rc) return rc;
  Upd U = upd_store(p);
  U.out = out;
  U.a = a;
  U.J = J;
  U.ja = ja;
  U.store = store;
  if (masked) {
    U.m0 = p->mask[0];
    U.m1 = p->mask[1];
    U.m2 = p->mask[2];
  }
  return run_line_pass<T>(p, 2, +1, 3, nullptr, W, U, s);
}

int curl_any(SbePstd3* p, const double2* F, double2* out, double a, const double2* J, double ja,
             bool masked, int store, cudaStream_t s) {
  return p->fp32 ? curl_pipeline<float2>(p, F, out, a, J, ja, masked, store, s)
                 : curl_pipeline<double2>(p, F, out, a, J, ja, masked, store, s);
}

bool is_masked(const SbePstd3* p) { return p->n_abc[0] > 0 || p->n_abc[1] > 0 || p->n_abc[2] > 0; }

// ---- the three-pass curl (FP32 work, planes in shared memory) -----------------
bool planes_fit(const SbePstd3* p) { return p->fp32 && (long long)p->n[1] * p->n[2] <= kPlaneMax; }

PlaneArgs plane_args(const SbePstd3* p) {
  PlaneArgs A{};
  A.nx = p->n[0];
  A.ny = p->n[1];
  A.nz = p->n[2];
  A.lgy = ilog2i(A.ny);
  A.lgz = ilog2i(A.nz);
  A.N = p->N;
  A.P = (long long)A.ny * A.nz;
  A.twy = p->twf[1];
  A.twz = p->twf[2];
  return A;
}

size_t plane_smem(const PlaneArgs& A) {
  return sizeof(float2) * ((size_t)plane_slots(A.P, A.lgz) + (A.ny >> 1) + (A.nz >> 1));
}

// x-pass columns per block: the three components' x lines of tl columns within
// kXSmem, tl <= 16 and dividing the plane
int x_lines(const SbePstd3* p) {
  const long long P = (long long)p->n[1] * p->n[2];
  int tl = 16;
  while (tl > 1 && ((size_t)3 * p->n[0] * tl * sizeof(float2) > (size_t)kXSmem || P % tl)) tl >>= 1;
  return tl;
}

int plane_pass_a(SbePstd3* p, const double2* F, cudaStream_t s) {
  const PlaneArgs A = plane_args(p);
  k_plane_fwd<<<dim3(A.nx, 3), kPlaneThreads, plane_smem(A), s>>>(A, F,
                                                                  static_cast<float2*>(p->work));
  return cuda_check(cudaGetLastError(), "pstd3 plane pass");
}

int plane_pass_b(SbePstd3* p, cudaStream_t s) {
  const PlaneArgs A = plane_args(p);
  const int tl = x_lines(p), nx = p->n[0];
  const size_t smem = sizeof(float2) * ((size_t)3 * nx * tl + (nx >> 1));
  k_x_curl_ip<<<(unsigned)(A.P / tl), kXThreads, smem, s>>>(
      A, static_cast<float2*>(p->work), ilog2i(nx), tl, p->twf[0], p->qb[0], p->qb[1], p->qb[2]);
  return cuda_check(cudaGetLastError(), "pstd3 x pass");
}

int plane_pass_c(SbePstd3* p, const Upd& U, int fwd_next, cudaStream_t s) {
  const PlaneArgs A = plane_args(p);
  k_plane_inv<<<dim3(A.nx, 3), kPlaneThreads, plane_smem(A), s>>>(
      A, static_cast<float2*>(p->work), U, fwd_next);
  return cuda_check(cudaGetLastError(), "pstd3 plane pass");
}

Upd upd_for(SbePstd3* p, double2* out, double a, const double2* J, double ja, bool masked,
            int store) {
  Upd U = upd_store(p);
  U.out = out;
  U.a = a;
  U.J = J;
  U.ja = ja;
  U.store = store;
  if (masked) {
    U.m0 = p->mask[0];
    U.m1 = p->mask[1];
    U.m2 = p->mask[2];
  }
  for (int ax = 0; ax < 3; ++ax) U.nabc[ax] = p->n_abc[ax];
  // FP32 pairs of the plane path: the curl arrives as N curl (N a power of two)
  const double an = (store ? 1.0 : a) / (double)p->N;
  U.af[0] = (float)an;
  U.af[1] = (float)(an - (double)U.af[0]);
  U.jf[0] = (float)ja;
  U.jf[1] = (float)(ja - (double)U.jf[0]);
  return U;
}

// out (+)= a curl F ...: the three-pass form when the planes fit, else five passes
int curl_best(SbePstd3* p, const double2* F, double2* out, double a, const double2* J, double ja,
              bool masked, int store, cudaStream_t s) {
  if (!planes_fit(p)) return curl_any(p, F, out, a, J, ja, masked, store, s);
  int rc = plane_pass_a(p, F, s);
  if (!rc) rc = plane_pass_b(p, s);
  if (!rc) rc = plane_pass_c(p, upd_for(p, out, a, J, ja, masked, store), 0, s);
  return rc;
}

}  // namespace

// The H half-step of a field step, leaving the work array ready for the E half-step
// of the same step: with planes in shared memory the H update's last pass continues
// with the first pass of curl H on the new H.
int pstd3_update_h_fwd(SbePstd3* p, const double2* E, double2* H, double dt, cudaStream_t s) {
  if (!planes_fit(p))
    return curl_any(p, E, H, -dt / kMu0, nullptr, 0.0, is_masked(p), 0, s);
  int rc = plane_pass_a(p, E, s);
  if (!rc) rc = plane_pass_b(p, s);
  if (!rc) rc = plane_pass_c(p, upd_for(p, H, -dt / kMu0, nullptr, 0.0, is_masked(p), 0), 1, s);
  return rc;
}

// The E half-step after pstd3_update_h_fwd on the same H, with nothing else using the
// work array in between.
int pstd3_update_e_from_work(SbePstd3* p, double2* E, const double2* H, const double2* J,
                             double dt, cudaStream_t s) {
  const double ie = dt / (kEps0 * p->epsr);
  if (!planes_fit(p)) return curl_any(p, H, E, ie, J, ie, is_masked(p), 0, s);
  int rc = plane_pass_b(p, s);
  if (!rc) rc = plane_pass_c(p, upd_for(p, E, ie, J, ie, is_masked(p), 0), 0, s);
  return rc;
}

}  // namespace sbe

using namespace sbe;

extern "C" {

int sbe_pstd3_create(const SbePstd3Desc* d, void* stream, SbePstd3** out) {
  if (!d || !out) return fail(SBE_ERR_ARG, "sbe_pstd3_create: null");
  *out = nullptr;
  for (int a = 0; a < 3; ++a) {
    if (!pow2(d->n[a]))
      return fail(SBE_ERR_UNSUPPORTED, "sbe_pstd3_create: every axis must be a power of two in "
                                       "[2, 1024]");
    if (!(d->d[a] > 0) || d->n_abc[a] < 0 || 2 * d->n_abc[a] > d->n[a])
      return fail(SBE_ERR_ARG, "sbe_pstd3_create: bad spacing or absorbing width");
  }
  if (!(d->epsr > 0) || d->abc_strength < 0) return fail(SBE_ERR_ARG, "sbe_pstd3_create: bad epsr");
  SbePstd3* p = new SbePstd3();
  for (int a = 0; a < 3; ++a) {
    p->n[a] = d->n[a];
    p->n_abc[a] = d->n_abc[a];
    p->d[a] = d->d[a];
  }
  p->fp32 = d->fp32_work ? 1 : 0;
  p->epsr = d->epsr;
  p->abc = d->abc_strength;
  p->N = (long long)p->n[0] * p->n[1] * p->n[2];
  size_t tab = 0;
  for (int a = 0; a < 3; ++a)
    tab += ((3 * sizeof(double) + sizeof(double2) + 2 * sizeof(float2)) * p->n[a] + 1536);
  // work: ten FP64 complex fields (the longitudinal-field spectra; the curl uses three)
  const size_t work = sizeof(double2) * 10 * (size_t)p->N;
  if (cudaMalloc(&p->arena, tab + work) != cudaSuccess) {
    delete p;
    return fail(SBE_ERR_OOM, "sbe_pstd3_create: device allocation");
  }
  char* b = static_cast<char*>(p->arena);
  auto take = [&](size_t bytes) {
    char* r = b;
    b += (bytes + 255) / 256 * 256;
    return r;
  };
  cudaStream_t s = as_stream(stream);
  for (int a = 0; a < 3; ++a) {
    const int n = p->n[a];
    p->x[a] = reinterpret_cast<double*>(take(sizeof(double) * n));
    p->q[a] = reinterpret_cast<double*>(take(sizeof(double) * n));
    p->mask[a] = reinterpret_cast<double*>(take(sizeof(double) * n));
    p->tw[a] = reinterpret_cast<double2*>(take(sizeof(double2) * n));
    p->twf[a] = reinterpret_cast<float2*>(take(sizeof(float2) * n));
    p->qb[a] = reinterpret_cast<float2*>(take(sizeof(float2) * n));
    k_tables3<<<(n + 127) / 128, 128, 0, s>>>(n, p->d[a], p->x[a], p->q[a], p->tw[a], p->twf[a],
                                             p->qb[a], p->mask[a], p->n_abc[a], p->abc);
  }
  p->work = take(work);
  int rc = cuda_check(cudaGetLastError(), "sbe_pstd3_create");
  if (!rc) {
    const int smem = kSmemMax + 1024;
    cudaFuncSetAttribute(k_line_pass<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_line_pass<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_x_curl<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_plane_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_plane_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_x_curl_ip, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    rc = cuda_check(cudaFuncSetAttribute(k_x_curl<float2>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                    "sbe_pstd3_create: shared memory");
  }
  if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "sbe_pstd3_create: tables");
  if (rc) {
    cudaFree(p->arena);
    delete p;
    return rc;
  }
  *out = p;
  return SBE_OK;
}

int sbe_pstd3_destroy(SbePstd3* p) {
  if (!p) return SBE_OK;
  cudaFree(p->arena);
  delete p;
  return SBE_OK;
}

int sbe_pstd3_grid(SbePstd3* p, int axis, double* x, double* q, void* stream) {
  if (!p || axis < 0 || axis > 2) return fail(SBE_ERR_ARG, "sbe_pstd3_grid: bad arguments");
  cudaStream_t s = as_stream(stream);
  const size_t b = sizeof(double) * p->n[axis];
  if (x) cudaMemcpyAsync(x, p->x[axis], b, cudaMemcpyDeviceToDevice, s);
  if (q) cudaMemcpyAsync(q, p->q[axis], b, cudaMemcpyDeviceToDevice, s);
  return cuda_check(cudaGetLastError(), "sbe_pstd3_grid");
}

int sbe_pstd3_curl(SbePstd3* p, const double* F, double* out, void* stream) {
  if (!p || !F || !out) return fail(SBE_ERR_ARG, "sbe_pstd3_curl: null");
  return curl_best(p, (const double2*)F, (double2*)out, 1.0, nullptr, 0.0, false, 1,
                   as_stream(stream));
}

int sbe_pstd3_update_h(SbePstd3* p, const double* E, double* H, double dt, void* stream) {
  if (!p || !E || !H) return fail(SBE_ERR_ARG, "sbe_pstd3_update_h: null");
  return curl_best(p, (const double2*)E, (double2*)H, -dt / kMu0, nullptr, 0.0, is_masked(p), 0,
                   as_stream(stream));
}

int sbe_pstd3_update_e(SbePstd3* p, double* E, const double* H, const double* J, double dt,
                       void* stream) {
  if (!p || !E || !H) return fail(SBE_ERR_ARG, "sbe_pstd3_update_e: null");
  const double ie = dt / (kEps0 * p->epsr);
  return curl_best(p, (const double2*)H, (double2*)E, ie, (const double2*)J, ie, is_masked(p), 0,
                   as_stream(stream));
}

int sbe_pstd3_step(SbePstd3* p, double* E, double* H, const double* J, double dt, void* stream) {
  if (!p) return fail(SBE_ERR_ARG, "sbe_pstd3_step: null");
  // stability of the spectral leapfrog: v dt |q|max / 2 <= 1
  const double v = 299792458.0 / std::sqrt(p->epsr);
  double qm = 0.0;
  for (int a = 0; a < 3; ++a) qm += (kPi / p->d[a]) * (kPi / p->d[a]);
  if (v * dt * std::sqrt(qm) / 2.0 > 1.0)
    return fail(SBE_ERR_ARG, "sbe_pstd3_step: dt above the stability limit 2 / (v |q|max)");
  if (!E || !H) return fail(SBE_ERR_ARG, "sbe_pstd3_step: null");
  cudaStream_t s = as_stream(stream);
  int rc = pstd3_update_h_fwd(p, (const double2*)E, (double2*)H, dt, s);
  if (rc) return rc;
  return pstd3_update_e_from_work(p, (double2*)E, (const double2*)H, (const double2*)J, dt, s);
}

// rhoPJ.py:703-880 ElongfromRho with the caller's wavenumber tables (the reference
// passes its centred GetKxArray/GetKyArray/GetKzArray, typespace.py:958-1030): FP64
// forward transforms of rho, Px, Py, Pz (P_k receives the transformed P, as the
// reference leaves it in its inputs; may be NULL), the k-space terms and ten FP64
// inverse transforms into out10 = [E_PRho x, y, z, E_P x, y, z, E_Rho x, y, z, rho_B].
int sbe_pstd3_elong(SbePstd3* p, const double* rho, const double* P3, const double* qx,
                    const double* qy, const double* qz, double* out10, double* P_k,
                    void* stream) {
  if (!p || !rho || !P3 || !qx || !qy || !qz || !out10)
    return fail(SBE_ERR_ARG, "sbe_pstd3_elong: null");
  cudaStream_t s = as_stream(stream);
  const long long N = p->N;
  double2* O = reinterpret_cast<double2*>(out10);
  // the four transforms in out10's first four fields (FP64 work: the reference's FFT)
  cudaMemcpyAsync(O, rho, sizeof(double2) * N, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(O + N, P3, sizeof(double2) * 3 * N, cudaMemcpyDeviceToDevice, s);
  Upd none = upd_store(p);
  int rc = SBE_OK;
  for (int a = 2; a >= 0 && !rc; --a) rc = run_line_pass<double2>(p, a, -1, 4, nullptr, O, none, s);
  if (rc) return rc;
  if (P_k) cudaMemcpyAsync(P_k, O + N, sizeof(double2) * 3 * N, cudaMemcpyDeviceToDevice, s);
  double2* S = static_cast<double2*>(p->work);
  cudaMemcpyAsync(S, O, sizeof(double2) * 4 * N, cudaMemcpyDeviceToDevice, s);
  double q01[2];
  rc = cuda_check(cudaMemcpyAsync(q01, qx, sizeof(double) * 2, cudaMemcpyDeviceToHost, s),
                  "sbe_pstd3_elong: q");
  if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "sbe_pstd3_elong: q");
  if (rc) return rc;
  const double small = (q01[1] - q01[0]) / 1e4;
  k_elong3<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(N, p->n[1], p->n[2], S, O, qx, qy, qz,
                                                       small, 1.0 / (kEps0 * p->epsr));
  // inverse transforms of the ten spectra; the last pass divides by N
  for (int a = 0; a < 2 && !rc; ++a) rc = run_line_pass<double2>(p, a, +1, 10, nullptr, O, none, s);
  if (rc) return rc;
  Upd U = upd_store(p);
  U.out = O;
  U.store = 1;
  // the last pass reads the work array: move the spectra there first
  cudaMemcpyAsync(S, O, sizeof(double2) * 10 * N, cudaMemcpyDeviceToDevice, s);
  rc = run_line_pass<double2>(p, 2, +1, 10, nullptr, S, U, s);
  return rc ? rc : cuda_check(cudaGetLastError(), "sbe_pstd3_elong");
}

}  // extern "C"
