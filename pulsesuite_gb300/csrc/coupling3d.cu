// Field <-> wire pieces of the 3-D coupling: CalcJfx (rhoPJ.py:491-515, free current
// from the change of the wire charge), QWPlacement (rhoPJ.py:655-702, the wire field
// spread onto the Maxwell grid through the gates gx gy gz) and EAtXYZ
// (usefulsubs.py:1996-2075 with locator :1803-1830, trilinear sampling of a grid
// field), here batched over any number of sample points.  Device pointers; complex
// arrays are interleaved c128.
#include <algorithm>
#include <cmath>

#include "sbe_ctx.cuh"
#include "sbe_gb300.h"
#include "sbe_internal.cuh"

namespace sbe {
namespace {

constexpr int kScanThreads = 1024;

// J[0] = 0, J[i] = J[i-1] - ((new_i - prev_i) / dt) dx: each thread runs the
// recurrence over its own contiguous chunk, a scan over the chunk totals gives the
// offsets, then every thread writes its chunk
__global__ void __launch_bounds__(kScanThreads) k_calc_jfx(long long n, const double2* rn,
                                                           const double2* rp, double dt,
                                                           double dx, double2* J) {
  __shared__ double2 tot[kScanThreads];
  const long long chunk = (n + kScanThreads - 1) / kScanThreads;
  const long long a0 = chunk * threadIdx.x, b0 = chunk * (threadIdx.x + 1);
  const long long a = a0 > 1 ? a0 : 1, b = b0 < n ? b0 : n;
  auto term = [&](long long i) {
    const double dr = (rn[i].x - rp[i].x) / dt, di = (rn[i].y - rp[i].y) / dt;
    return make_double2(__dmul_rn(dr, dx), __dmul_rn(di, dx));
  };
  double2 s = make_double2(0.0, 0.0);
  for (long long i = a; i < b; ++i) {
    const double2 t = term(i);
    s.x = __dsub_rn(s.x, t.x);
    s.y = __dsub_rn(s.y, t.y);
  }
  tot[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 run = make_double2(0.0, 0.0);
    for (int t = 0; t < kScanThreads; ++t) {
      const double2 v = tot[t];
      tot[t] = run;
      run.x += v.x;
      run.y += v.y;
    }
  }
  __syncthreads();
  double2 acc = tot[threadIdx.x];
  if (threadIdx.x == 0 && n > 0) J[0] = make_double2(0.0, 0.0);
  for (long long i = a; i < b; ++i) {
    const double2 t = term(i);
    acc.x = __dsub_rn(acc.x, t.x);
    acc.y = __dsub_rn(acc.y, t.y);
    J[i] = acc;
  }
}

// Fgrid[i][j][k] = 0 + gx_i gy_j gz_k Fwire_i (C order, k fastest)
__global__ void k_qw_placement(int nx, int ny, int nz, const double2* fw, const double* gx,
                               const double* gy, const double* gz, double2* grid) {
  const long long tot = (long long)nx * ny * nz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e % nz);
    const long long ij = e / nz;
    const int j = (int)(ij % ny), i = (int)(ij / ny);
    const double g = __dmul_rn(__dmul_rn(gx[i], gy[j]), gz[k]);
    grid[e] = make_double2(__dadd_rn(0.0, __dmul_rn(g, fw[i].x)),
                           __dadd_rn(0.0, __dmul_rn(g, fw[i].y)));
  }
}

// locator: searchsorted(x, x0, 'right') - 1 clamped to [0, n - 2]
__device__ int locate(const double* x, int n, double x0) {
  int lo = 0, hi = n;   // first index with x > x0
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] <= x0) lo = mid + 1;
    else hi = mid;
  }
  const int i = lo - 1 < n - 2 ? lo - 1 : n - 2;
  return i > 0 ? i : 0;
}

__device__ void axis(const double* x, int n, double x0, int* i, double w[2]) {
  if (n == 1) {
    *i = 0;
    w[0] = 1.0;
    w[1] = 0.0;
    return;
  }
  *i = locate(x, n, x0);
  const double al = __ddiv_rn(x0 - x[*i], x[*i + 1] - x[*i]);
  w[0] = 1.0 - al;
  w[1] = al;
}

__global__ void k_e_at_xyz(const double2* f, const double* x, int nx, const double* y, int ny,
                           const double* z, int nz, const double* pts, int npts, double2* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  int i, j, k;
  double wx[2], wy[2], wz[2];
  axis(x, nx, pts[3 * p], &i, wx);
  axis(y, ny, pts[3 * p + 1], &j, wy);
  axis(z, nz, pts[3 * p + 2], &k, wz);
  double2 f0 = make_double2(0.0, 0.0);
  for (int r = 0; r < 2; ++r)
    for (int q = 0; q < 2; ++q)
      for (int s = 0; s < 2; ++s) {
        // a singleton axis has weight 0 on its second point, which does not exist
        if ((s && nx == 1) || (q && ny == 1) || (r && nz == 1)) continue;
        const double w = __dmul_rn(__dmul_rn(wx[s], wy[q]), wz[r]);
        const double2 v = f[((long long)(i + s) * ny + (j + q)) * nz + (k + r)];
        f0.x = __dadd_rn(f0.x, __dmul_rn(w, v.x));
        f0.y = __dadd_rn(f0.y, __dmul_rn(w, v.y));
      }
  out[p] = f0;
}

}  // namespace
}  // namespace sbe

using namespace sbe;

extern "C" int sbe_calc_jfx(long long n, const double* rho_new, const double* rho_prev, double dt,
                            double dx, double* J, void* stream) {
  if (n < 0 || (n > 0 && (!rho_new || !rho_prev || !J)) || dt == 0.0)
    return fail(SBE_ERR_ARG, "sbe_calc_jfx: bad arguments");
  if (n == 0) return SBE_OK;
  k_calc_jfx<<<1, kScanThreads, 0, (cudaStream_t)stream>>>(
      n, (const double2*)rho_new, (const double2*)rho_prev, dt, dx, (double2*)J);
  return cuda_check(cudaGetLastError(), "sbe_calc_jfx");
}

extern "C" int sbe_qw_placement(int nx, int ny, int nz, const double* Fwire, const double* gx,
                                const double* gy, const double* gz, double* Fgrid, void* stream) {
  if (nx < 0 || ny < 0 || nz < 0 || !Fwire || !gx || !gy || !gz || !Fgrid)
    return fail(SBE_ERR_ARG, "sbe_qw_placement: bad arguments");
  const long long tot = (long long)nx * ny * nz;
  if (tot == 0) return SBE_OK;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (tot + 255) / 256;
  const int blocks = (int)std::min<long long>(want, (long long)std::max(sms, 1) * 8);
  k_qw_placement<<<blocks, 256, 0, (cudaStream_t)stream>>>(nx, ny, nz, (const double2*)Fwire, gx,
                                                           gy, gz, (double2*)Fgrid);
  return cuda_check(cudaGetLastError(), "sbe_qw_placement");
}

extern "C" int sbe_e_at_xyz(const double* f, const double* x, int nx, const double* y, int ny,
                            const double* z, int nz, const double* pts, int npts, double* out,
                            void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || npts < 0 || !f || !x || !y || !z ||
      (npts > 0 && (!pts || !out)))
    return fail(SBE_ERR_ARG, "sbe_e_at_xyz: bad arguments");
  if (npts == 0) return SBE_OK;
  k_e_at_xyz<<<(npts + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      (const double2*)f, x, nx, y, ny, z, nz, pts, npts, (double2*)out);
  return cuda_check(cudaGetLastError(), "sbe_e_at_xyz");
}
