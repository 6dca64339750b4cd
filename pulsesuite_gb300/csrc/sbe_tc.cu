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
    double vr = v.x * sc, vi = v.y * sc;
    __half rh = __double2half(vr);
    __half rl = __double2half(vr - (double)__half2float(rh));
    base[o] = rh;
    base[plane + o] = rl;
    if (!real_only) {
      __half ih = __double2half(vi);
      __half il = __double2half(vi - (double)__half2float(ih));
      base[2 * plane + o] = ih;
      base[3 * plane + o] = il;
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

void mixed_free(SbeCtx* c) { (void)c; }

int rhs_mixed(SbeCtx* c, const double2* P, const double2* C, const double2* D, double2* dP,
              double2* dC, double2* dD, cudaStream_t s) {
  (void)c; (void)P; (void)C; (void)D; (void)dP; (void)dC; (void)dD; (void)s;
  return fail(SBE_ERR_UNSUPPORTED, "mixed precision path not built");
}

int rk4_mixed(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek0,
              const double2* dEk, double dt, double2* src, cudaStream_t s) {
  (void)c; (void)P; (void)C; (void)D; (void)Ek0; (void)dEk; (void)dt; (void)src; (void)s;
  return fail(SBE_ERR_UNSUPPORTED, "mixed precision path not built");
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
