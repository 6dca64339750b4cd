// Mixed-precision (tcgen05) path of the SBE right-hand side: FP16 hi/lo plane
// conversion, per-wire power-of-two scaling, the stage pipeline and the
// self-test entry point.
//
// GB300 executes FP64 arithmetic and the double <-> float conversions at a
// small fraction of its FP32 rate, so the per-element code of this file uses
// FP32 arithmetic and the integer-pipe conversions of fp_bits.cuh.  FP64
// arithmetic is kept where the result needs it: the RK4 accumulation of the
// state and the peeled diagonal energies (formed once per row).
#include <cuda_fp16.h>

#include <algorithm>
#include <vector>

#include "fp_bits.cuh"
#include "sbe_ctx.cuh"
#include "tc_gemm.cuh"
#include "sbe_mixed.cuh"

namespace sbe {

// ---------------------------------------------------------------------------
// max(|re|, |im|) of each batch entry of a packed complex array (integer compare
// of the magnitudes' bit patterns; atomicMax on the pattern of the FP32 value).
__global__ void k_absmax(const double2* X, long long per_batch, long long bstride, unsigned* out) {
  const int b = blockIdx.y;
  const double2* x = X + (long long)b * bstride;
  unsigned long long m = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per_batch;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 v = x[i];
    m = max(m, max(absbits(v.x), absbits(v.y)));
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out + b, bits_to_fmax(m));
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

// The exponents of one stage in one launch (one thread per wire): eS from the
// full state maximum, eO from the off-diagonal one, esx = eT + eS (exchange
// products); with reset set the maxima are cleared for the fused RK4 update of
// the stage, which collects the next state's maxima in them; mxH is cleared for
// the stage's Hamiltonian.
__global__ void k_stage_exponents(int nb, unsigned* mxS, unsigned* mxO, unsigned* mxH, int* eS,
                                  int* eO, const int* eT, int* esx, int reset) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float ms = __uint_as_float(mxS[b]) * 1.0001f, mo = __uint_as_float(mxO[b]) * 1.0001f;
  const int vs = (ms > 0.f) ? 14 - (int)ceilf(log2f(ms)) : 0;
  eS[b] = vs;
  eO[b] = (mo > 0.f) ? 14 - (int)ceilf(log2f(mo)) : 0;
  esx[b] = eT[b] + vs;
  mxH[b] = 0u;
  if (reset) {
    mxS[b] = 0u;
    mxO[b] = 0u;
  }
}

// e[b] from the larger of two maxima (rule of k_exponents) and sum[b] = e[b] + add[b]
__global__ void k_exponents2_sum(int nb, const unsigned* mx1, const unsigned* mx2, int* e,
                                 const int* add, int* sum) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float m = fmaxf(__uint_as_float(mx1[b]), __uint_as_float(mx2[b])) * 1.0001f;
  const int v = (m > 0.f) ? 14 - (int)ceilf(log2f(m)) : 0;
  e[b] = v;
  sum[b] = v + add[b];
}

__device__ __forceinline__ void put_hilo(__half* base, long long plane, float v) {
  const __half h = __float2half_rn(v);
  base[0] = h;
  base[plane] = __float2half_rn(v - __half2float(h));
}

// FP16 hi/lo planes of a batch of Nk x Nk complex matrices, scaled by 2^e[b];
// optionally transposed.  dst layout [mat][plane][batch][rows][K]; planes
// re_hi, re_lo, im_hi, im_lo (complex) or hi, lo of the real part.
__global__ void k_planes(const double2* X, long long bstride, int nk, int transpose,
                         const int* e, tc::PlaneSet dst, int mat, int real_only) {
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
  const int eb = e[b];
  const long long pstride = (long long)dst.batch * tc::plane_slab(dst);   // next plane
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int r = r0 + i, c = c0 + threadIdx.x;
    if (r >= nk || c >= nk) continue;
    double2 v = transpose ? tile[threadIdx.x][i] : tile[i][threadIdx.x];
    __half* base = dst.ptr + tc::plane_elem(dst, mat, 0, b, r, c);
    // exact scaling and one rounding to FP32 (24 bits >= the 22 the planes keep)
    put_hilo(base, pstride, f64_to_f32(v.x, eb));
    if (!real_only) put_hilo(base + 2 * pstride, pstride, f64_to_f32(v.y, eb));
  }
}

void launch_planes(const double2* X, long long bstride, int nk, int nbatch, int transpose,
                   const int* e, const tc::PlaneSet& dst, int mat, int real_only,
                   cudaStream_t s) {
  dim3 blk(32, 8), grid((nk + 31) / 32, (nk + 31) / 32, nbatch);
  k_planes<<<grid, blk, 0, s>>>(X, bstride, nk, transpose, e, dst, mat, real_only);
}

// a complex value scaled by 2^e and rounded once to FP32
template <typename T>
__device__ __forceinline__ float2 scaled2(T v, int e);
template <>
__device__ __forceinline__ float2 scaled2<double2>(double2 v, int e) {
  return f64_to_f32(v, e);
}
template <>
__device__ __forceinline__ float2 scaled2<float2>(float2 v, int e) {
  return make_float2(f32_ldexp(v.x, e), f32_ldexp(v.y, e));
}

// With cdf set, the diagonal is left out of the planes (written as zero) and the
// hi / lo FP32 parts of its real part (from dg[b * nk + k] in FP64 when given) go
// to cdf[b * nk + k] and cdf[nbatch * nk + b * nk + k].
__device__ __forceinline__ double dvalue(double2 v) { return v.x; }
__device__ __forceinline__ double dvalue(float2 v) { return f32_to_f64(v.x); }

// FP16 hi / lo of one FP32 value pair (re, im): planes re_hi, re_lo, im_hi, im_lo
__device__ __forceinline__ void hilo4(float2 v, __half* h0, __half* h1, __half* h2, __half* h3) {
  const __half2 hi = __float22half2_rn(v);
  const float2 hf = __half22float2(hi);
  const __half2 lo = __float22half2_rn(make_float2(v.x - hf.x, v.y - hf.y));
  *h0 = __low2half(hi);
  *h1 = __low2half(lo);
  *h2 = __high2half(hi);
  *h3 = __high2half(lo);
}

// Store the 32 x 32 plane tiles hs[plane][row][k] (row stride 40 halves) of rows
// r0.., K-block kb: four lanes write the 64 bytes of one row (16-byte stores).
__device__ __forceinline__ void store_tiles(const __half (*hs)[32][40], int npl,
                                            const tc::PlaneSet& dst, int mat, int b, int r0,
                                            int kb, int tid, int nthreads) {
  for (int t = tid; t < npl * 128; t += nthreads) {
    const int pl = t >> 7, rr = (t >> 2) & 31, j = t & 3;
    const uint4 v = *reinterpret_cast<const uint4*>(&hs[pl][rr][8 * j]);
    *reinterpret_cast<uint4*>(dst.ptr + tc::chunk_elem(dst, mat, pl, b, r0 + rr, kb, j)) = v;
  }
}

// The same tiles transposed: row r0 + cc of the destination holds column cc of hs.
__device__ __forceinline__ void store_tiles_t(const __half (*hs)[32][40], int npl,
                                              const tc::PlaneSet& dst, int mat, int b, int r0,
                                              int kb, int tid, int nthreads) {
  for (int t = tid; t < npl * 128; t += nthreads) {
    const int pl = t >> 7, cc = (t >> 2) & 31, j = t & 3;
    __align__(16) __half v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = hs[pl][8 * j + i][cc];
    *reinterpret_cast<uint4*>(dst.ptr + tc::chunk_elem(dst, mat, pl, b, r0 + cc, kb, j)) =
        *reinterpret_cast<const uint4*>(v);
  }
}

// Both layouts of a batch of Nk x Nk complex matrices from one read: planes of X
// into matrix slot matN and of X^T into slot matT (matT < 0: none), same scale.
// The block (32 x 8 threads) converts its 32 x 32 tile once into shared-memory
// plane tiles and writes both layouts with 16-byte stores.
template <typename T>
__global__ void k_planes_nt(const T* X, int nk, const int* e, tc::PlaneSet dst, int matN, int matT,
                            int nbatch, float* cdf = nullptr, const double* dg = nullptr) {
  __shared__ T tile[32][33];
  __shared__ __align__(16) __half hs[4][32][40];
  const int b = blockIdx.z;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const T* x = X + (long long)b * nk * nk;
  {
    // block (32, 8): four rows per thread, all loads issued before the stores
    T v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int r = r0 + threadIdx.y + 8 * k, c = c0 + threadIdx.x;
      T z;
      z.x = 0;
      z.y = 0;
      v[k] = (r < nk && c < nk) ? x[(long long)r * nk + c] : z;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) tile[threadIdx.y + 8 * k][threadIdx.x] = v[k];
  }
  __syncthreads();
  const int eb = e[b];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = threadIdx.y + 8 * k;
    const int r = r0 + i, c = c0 + threadIdx.x;
    float2 v = scaled2<T>(tile[i][threadIdx.x], eb);
    if (cdf && r == c && r < nk) {
      v = make_float2(0.f, 0.f);
      const double d = dg ? dg[(long long)b * nk + r] : dvalue(tile[i][threadIdx.x]);
      const float hi = f64_to_f32(d);
      cdf[(long long)b * nk + r] = hi;
      cdf[((long long)nbatch + b) * nk + r] = f64_to_f32(d - f32_to_f64(hi));
    }
    hilo4(v, &hs[0][i][threadIdx.x], &hs[1][i][threadIdx.x], &hs[2][i][threadIdx.x],
          &hs[3][i][threadIdx.x]);
  }
  __syncthreads();
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
  store_tiles(hs, 4, dst, matN, b, r0, c0 >> 5, tid, nth);
  if (matT >= 0) store_tiles_t(hs, 4, dst, matT, b, c0, r0 >> 5, tid, nth);
}

// Band of the sheared state planes (k_shear_tiles): the first dd block of the
// t' block at t0 whose source rows can reach the matrix, and whether the block
// (t0, dd0) holds any element of it.
__host__ __device__ inline int shear_first_block(int nk, int t0) {
  const int lo = nk - 63 - t0;   // lowest dd whose 63 source rows reach row 0
  return lo > 0 ? lo / 32 : 0;
}
__host__ __device__ inline bool shear_block_live(int nk, int t0, int dd0) {
  const int rbase = t0 + dd0 - (nk - 1);
  return rbase + 62 >= 0 && rbase < nk;
}

// Traces from the diagonal partials of k_shear_tiles: diagonal dd = k1 - k2 + Nk - 1
// of X (row k1, column k2) is trace index d + Nk with d = k2 - k1, summed over the
// nb column blocks in a fixed order into trf[b][which][d + Nk] (SBEs.py:1094-1103).
__global__ void k_trace_from_shear(int nk, int nb, int ndd, const float2* dpart, float2* trf) {
  const int b = blockIdx.z, which = blockIdx.y;
  const int dd = blockIdx.x * blockDim.x + threadIdx.x;
  if (dd >= 2 * nk - 1) return;
  const float2* part = dpart + (((long long)b * 2 + which) * ndd + dd) * nb;
  float sr = 0.f, si = 0.f;
  for (int i = 0; i < nb; ++i) {
    if (!shear_block_live(nk, 32 * i, dd & ~31)) continue;   // no block, all zero
    const float2 v = part[i];
    sr += v.x;
    si += v.y;
  }
  trf[(long long)b * 4 * nk + which * 2 * nk + (2 * nk - 1 - dd)] = make_float2(sr, si);
}

void launch_exponents(const double2* X, long long per_batch, long long bstride, int nbatch,
                      unsigned* mx, int* e, const int* add, int* sum, cudaStream_t s) {
  cudaMemsetAsync(mx, 0, sizeof(unsigned) * nbatch, s);
  int blocks = (int)std::min<long long>((per_batch + 255) / 256, 256);
  k_absmax<<<dim3(blocks, nbatch), 256, 0, s>>>(X, per_batch, bstride, mx);
  k_exponents<<<(nbatch + 127) / 128, 128, 0, s>>>(nbatch, mx, e, add, sum);
}

// ---------------------------------------------------------------------------
// Mixed-precision workspace of a context.  The layout groups the wires by Nk, so
// the wires of one Nk form a bucket whose matrices are one contiguous block of
// every packed buffer: the per-element kernels run once per bucket (uniform Nk,
// grid z = the bucket's wires) on pointers offset to the bucket's block, and each
// GEMM kind runs as one persistent launch over the jobs of all buckets.
//
// Per bucket, commutator planes: 14 matrix slots x 4 planes x Nw x Nk x Nk (FP16):
//   0 P, 1 P^T, 2 C, 4 D                            (state, exponent eS)
//   6 Heh, 7 Heh^T, 8 Hee', 10 Hhh',
//   12 Hee' + i hbar B, 13 Hhh' + i hbar A          (Hamiltonians, exponent eH)
// (' = diagonal removed; A, B = off-diagonal dephasing matrices; C^T = conj C and
// D^T = conj D are taken by conjugating the C and D operands).
// Exchange: Toeplitz planes T_n (3 x 2 x Nw x Nk x Nk) and sheared state planes
// S_n (3 x 2 x Nw x 4Nk x Nk).  Sources: E^T planes (4 x Nw x Nr x Nk).
// Context-wide FP32 stage values (indexed like the packed state): kf (dP, dC, dD),
// accf (RK4 sums), hf (Heh, Hee', Hhh'), habf (hbar A, hbar B), the phonon tables,
// the stage field and Expikr.
void mixed_free(SbeCtx* c) {
  MixedAll* A = all_of(c);
  if (!A) return;
  for (Mixed* m : A->b) {
    cudaFree(m->pl.ptr);
    cudaFree(m->tp.ptr);
    cudaFree(m->sp.ptr);
    cudaFree(m->ep.ptr);
    cudaFree(m->xsh);
    cudaFree(m->block);
    cudaFree(m->dw);
    delete m;
  }
  cudaFree(A->block);
  delete A;
  c->mixed = nullptr;
}

// E^T planes: Y[r][k] = Expikr[k][r] (|E| = 1, exponent 13).
__global__ void k_eplanes(const WireDev* wires, const double2* expikr, tc::PlaneSet dst, int nw) {
  const WireDev W = wires[blockIdx.z];
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  int r = blockIdx.y;
  if (k >= W.nk || r >= W.nr) return;
  double2 v = expikr[W.off_kr + (long long)k * W.nr + r];
  const long long pstride = (long long)dst.batch * tc::plane_slab(dst);
  __half* base = dst.ptr + tc::plane_elem(dst, 0, 0, blockIdx.z, r, k);
  put_hilo(base, pstride, f64_to_f32(v.x, 13));
  put_hilo(base + 2 * pstride, pstride, f64_to_f32(v.y, 13));
}

__global__ void k_fill_int(int* p, int n, int v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// real absmax per wire of a packed Nk x Nk real table, as the FP64 bit pattern
// (the phonon tables exceed the FP32 range)
__global__ void k_absmax_r(const double* X, long long per, unsigned long long* out) {
  const int b = blockIdx.y;
  const double* x = X + (long long)b * per;
  unsigned long long m = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per;
       i += (long long)gridDim.x * blockDim.x)
    m = max(m, absbits(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out + b, m);
}

// sP[b] = -(E + 1) for max |EP|, |HP| in [2^E, 2^(E+1)): the scaled tables lie
// in [0, 1)
__global__ void k_phon_exp(int nb, const unsigned long long* mx, int* sP) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const unsigned long long m = mx[b];
  const int ex = (int)((m >> 52) & 0x7FF);
  sP[b] = (ex == 0) ? 0 : -((ex - 1023) + 1);
}

// EP, EP^T, HP, HP^T of every wire as scaled FP32 (coalesced transposes via tiles)
__global__ void k_phon_tables(int nk, const double* EP, const double* HP, const int* sP,
                              float* epf, float* eptf, float* hpf, float* hptf) {
  __shared__ double te[32][33], th[32][33];
  const int b = blockIdx.z;
  const long long mb = (long long)b * nk * nk;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int e = sP[b];
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    const bool ok = r < nk && c < nk;
    const double ve = ok ? EP[mb + (long long)r * nk + c] : 0.0;
    const double vh = ok ? HP[mb + (long long)r * nk + c] : 0.0;
    te[i][threadIdx.x] = ve;
    th[i][threadIdx.x] = vh;
    if (ok) {
      epf[mb + (long long)r * nk + c] = f64_to_f32(ve, e);
      hpf[mb + (long long)r * nk + c] = f64_to_f32(vh, e);
    }
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = c0 + i, c = r0 + threadIdx.x;   // row c0 + i of the transpose
    if (r < nk && c < nk) {
      eptf[mb + (long long)r * nk + c] = f64_to_f32(te[threadIdx.x][i], e);
      hptf[mb + (long long)r * nk + c] = f64_to_f32(th[threadIdx.x][i], e);
    }
  }
}

__global__ void k_ekrf(long long n, const double2* expikr, float2* ekrf) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) ekrf[i] = f64_to_f32(expikr[i]);
}

// |xe|, |xh| of a bucket's wires in FP32: xef[b][j], j < 2 nk
__global__ void k_xef(const WireDev* wires, int nk, const double* xeh, float* xef) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
  if (j < 2 * nk) xef[(long long)b * 2 * nk + j] = fabsf(f64_to_f32(xeh[2 * wires[b].off_vec + j]));
}

// carve 256-byte aligned parts out of one allocation
struct Carver {
  size_t off = 0;
  char* base = nullptr;
  template <typename T>
  T* take(size_t n) {
    const size_t o = off;
    off = (off + sizeof(T) * n + 255) / 256 * 256;
    return base ? reinterpret_cast<T*>(base + o) : nullptr;
  }
};

static void carve_bucket(Mixed* m, Carver& k) {
  const size_t v = (size_t)m->nw * m->nk;
  const int T = (m->nk + 31) / 32;
  m->ints = k.take<int>(9 * (size_t)m->nw);
  m->mx = k.take<unsigned>(4 * (size_t)m->nw);
  m->mx64 = k.take<unsigned long long>((size_t)m->nw);
  m->sP = k.take<int>((size_t)m->nw);
  m->vsf = k.take<float>(3 * v);
  m->trf = k.take<float2>(4 * v);
  m->gamf = k.take<float>(2 * v);
  m->dgf = k.take<float2>(4 * v);
  m->dgE = k.take<double2>(2 * v);
  m->dgH = m->dgE ? m->dgE + v : nullptr;
  m->xef = k.take<float>(2 * v);
  m->phf = k.take<float>(2 * v);
  m->gtab = k.take<float>(4 * v);
  m->tpart = k.take<float2>((size_t)m->nw * 2 * 32 * ((2 * m->nk + 31) / 32) * T);
  m->cdf = k.take<float>(4 * v);
  m->xdg = k.take<double>(2 * v);
}

static void carve_all(MixedAll* A, Carver& k, const SbeCtx* c) {
  const size_t tm = (size_t)c->tot_mat;
  A->kf = k.take<float2>(3 * tm);
  A->accf = k.take<float2>(3 * tm);
  A->hf = k.take<float2>(3 * tm);
  A->habf = k.take<float>(2 * tm);
  A->epf = k.take<float>(tm);
  A->eptf = k.take<float>(tm);
  A->hpf = k.take<float>(tm);
  A->hptf = k.take<float>(tm);
  A->ekf = k.take<float2>(3 * (size_t)c->tot_r);
  A->ekrf = k.take<float2>((size_t)c->tot_kr);
  A->err = k.take<int>(1);
}

static int mixed_ensure(SbeCtx* c, cudaStream_t s) {
  if (c->mixed) return SBE_OK;
  const int flags0 = c->wires[0].flags;
  for (int w = 1; w < c->nw; ++w)
    if (c->wires[w].flags != flags0)
      return fail(SBE_ERR_UNSUPPORTED,
                  "mixed path: all wires of a context must share their flags (one context per "
                  "flag set)");
  // the operand planes take C^T = conj C, D^T = conj D; the reference's DC transport
  // (dcfield.py:1196-1206: the centred Y against the FFT's natural order) leaves C, D
  // non-Hermitian, so DCTrans runs on the FP64 path only
  if (any_dc(c))
    return fail(SBE_ERR_UNSUPPORTED,
                "mixed path: DCTrans leaves C and D non-Hermitian; use the FP64 path");
  for (const auto& W : c->wires)
    if (W.nk % 8) return fail(SBE_ERR_UNSUPPORTED, "mixed path: Nk must be a multiple of 8");
  MixedAll* A = new MixedAll();
  c->mixed = A;
  // buckets: runs of equal Nk in the layout order
  for (int i = 0; i < c->nw;) {
    const WireDev& W0 = c->wires[c->order[i]];
    int j = i;
    while (j < c->nw && c->wires[c->order[j]].nk == W0.nk) ++j;
    Mixed* m = new Mixed();
    m->nk = W0.nk;
    m->nw = j - i;
    m->nr = 2 * W0.nk + 2;
    m->first = i;
    m->bm = W0.off_mat;
    m->bv = W0.off_vec;
    m->br = W0.off_r;
    m->bkr = W0.off_kr;
    // K parts of 128 or fewer from Nk = 256 on (four, eight from Nk = 1024): the
    // hi*hi chains of long K ranges set the truncation error of W - W^H (the
    // autotuner's cache may override)
    m->hs = W0.nk >= 1024 ? 8 : (W0.nk >= 256 ? 4 : 2);
    A->b.push_back(m);
    i = j;
  }
  bool ok = true;
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    const size_t mm = (size_t)nk * nk;
    m->pl = tc::make_planeset(nullptr, 14, 4, nw, nk, nk);
    m->tp = tc::make_planeset(nullptr, 3, 2, nw, nk, nk);
    m->sp = tc::make_planeset(nullptr, 3, 2, nw, 4 * nk, nk);
    m->ep = tc::make_planeset(nullptr, 1, 4, nw, m->nr, nk);
    Carver k;
    carve_bucket(m, k);
    const size_t vbytes = k.off;
    ok = ok && cudaMalloc(&m->pl.ptr, tc::planeset_bytes(m->pl)) == cudaSuccess &&
         cudaMalloc(&m->tp.ptr, tc::planeset_bytes(m->tp)) == cudaSuccess &&
         cudaMalloc(&m->sp.ptr, tc::planeset_bytes(m->sp)) == cudaSuccess &&
         cudaMalloc(&m->ep.ptr, tc::planeset_bytes(m->ep)) == cudaSuccess &&
         cudaMalloc(&m->xsh, sizeof(float) * 3 * nw * 2 * mm) == cudaSuccess &&
         cudaMalloc(&m->block, vbytes) == cudaSuccess &&
         cudaMalloc(&m->dw, sizeof(WireDev) * nw) == cudaSuccess;
    if (!ok) break;
    k = Carver{0, static_cast<char*>(m->block)};
    carve_bucket(m, k);
    std::vector<WireDev> hw(nw);
    for (int b = 0; b < nw; ++b) hw[b] = c->wires[c->order[m->first + b]];
    cudaMemcpyAsync(m->dw, hw.data(), sizeof(WireDev) * nw, cudaMemcpyHostToDevice, s);
    // the host vector goes out of scope: wait for the copy
    cudaStreamSynchronize(s);
  }
  Carver ka;
  carve_all(A, ka, c);
  ok = ok && cudaMalloc(&A->block, ka.off) == cudaSuccess;
  if (!ok) {
    mixed_free(c);
    return fail(SBE_ERR_OOM, "mixed path: workspace allocation failed");
  }
  ka = Carver{0, static_cast<char*>(A->block)};
  carve_all(A, ka, c);
  cudaMemsetAsync(A->block, 0, ka.off, s);
  k_ekrf<<<(unsigned)((c->tot_kr + 255) / 256), 256, 0, s>>>(c->tot_kr, c->expikr, A->ekrf);
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    const long long mm = (long long)nk * nk;
    const int T = (nk + 31) / 32;
    cudaMemsetAsync(m->ints, 0, sizeof(int) * 9 * nw, s);
    cudaMemsetAsync(m->mx, 0, sizeof(unsigned) * 4 * nw, s);
    // the padding of every plane set stays zero: producers write only inside; the
    // sheared planes are zeroed once, stages write only the in-band part
    cudaMemsetAsync(m->pl.ptr, 0, tc::planeset_bytes(m->pl), s);
    cudaMemsetAsync(m->tp.ptr, 0, tc::planeset_bytes(m->tp), s);
    cudaMemsetAsync(m->sp.ptr, 0, tc::planeset_bytes(m->sp), s);
    cudaMemsetAsync(m->ep.ptr, 0, tc::planeset_bytes(m->ep), s);
    k_eplanes<<<dim3((nk + 127) / 128, m->nr, nw), 128, 0, s>>>(m->dw, c->expikr, m->ep, nw);
    k_fill_int<<<(nw + 127) / 128, 128, 0, s>>>(m->eE(), nw, 13);
    cudaMemsetAsync(m->mx64, 0, sizeof(unsigned long long) * nw, s);
    k_absmax_r<<<dim3(64, nw), 256, 0, s>>>(c->EP + m->bm, mm, m->mx64);
    k_absmax_r<<<dim3(64, nw), 256, 0, s>>>(c->HP + m->bm, mm, m->mx64);
    k_phon_exp<<<(nw + 127) / 128, 128, 0, s>>>(nw, m->mx64, m->sP);
    k_phon_tables<<<dim3(T, T, nw), dim3(32, 8), 0, s>>>(nk, c->EP + m->bm, c->HP + m->bm, m->sP,
                                                        A->epf + m->bm, A->eptf + m->bm,
                                                        A->hpf + m->bm, A->hptf + m->bm);
    k_xef<<<dim3((2 * nk + 127) / 128, nw), 128, 0, s>>>(m->dw, nk, c->xeh, m->xef);
  }
  return cuda_check(cudaGetLastError(), "mixed workspace");
}

// maxima of a batch of Nk x Nk matrices: all elements into mx[b], and (when
// peel) the off-diagonal elements into mo[b] (all elements when !peel)
// Stage-1 state of the mixed path: the FP32 copy xf of a batch of Nk x Nk FP64
// matrices (round to nearest; every stage consumer rounds the state to FP32),
// its maxima mx (all elements) and mo (off-diagonal only when peel), and with dg
// set the FP64 real diagonal (the occupations of C and D, which the peeled terms
// use beyond FP32).  The diagonal is tracked by a row / column counter stepped
// with the grid stride (no division per element).
__global__ void __launch_bounds__(256) k_state_in(const double2* __restrict__ X, int nk, int peel,
                                                  unsigned* __restrict__ mx,
                                                  unsigned* __restrict__ mo,
                                                  float2* __restrict__ xf, double* __restrict__ dg) {
  const int b = blockIdx.y;
  const int per = nk * nk;   // < 2^31
  const double2* x = X + (long long)b * per;
  float2* y = xf + (long long)b * per;
  unsigned m = 0, o = 0;   // FP32 magnitude patterns
  // four elements per thread and pass (stride S), loads issued together; the
  // diagonal is tracked by row / column counters stepped with S (no division per
  // element)
  const int S = gridDim.x * blockDim.x;
  const int srow = S / nk, scol = S % nk;
  const int i00 = blockIdx.x * blockDim.x + threadIdx.x;
  int row = i00 / nk, col = i00 % nk;
  for (int i0 = i00; i0 < per; i0 += 4 * S) {
    double2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * S;
      v[u] = i < per ? x[i] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * S;
      if (i < per) {
        const float2 f = f64_to_f32(v[u]);
        y[i] = f;
        const unsigned a = max(__float_as_uint(f.x) & 0x7FFFFFFFu, __float_as_uint(f.y) & 0x7FFFFFFFu);
        m = max(m, a);
        const bool diag = row == col;
        if (diag && dg) dg[(long long)b * nk + row] = v[u].x;
        if (!(diag && peel)) o = max(o, a);
      }
      col += scol;
      row += srow;
      if (col >= nk) {
        col -= nk;
        ++row;
      }
    }
  }
  // one atomic pair per block: same-address atomics of all blocks serialise in L2
  __shared__ unsigned red[2][8];
  for (int k = 16; k > 0; k >>= 1) {
    m = max(m, __shfl_down_sync(0xffffffffu, m, k));
    o = max(o, __shfl_down_sync(0xffffffffu, o, k));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = m;
    red[1][threadIdx.x >> 5] = o;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      m = max(m, red[0][w]);
      o = max(o, red[1][w]);
    }
    atomicMax(mx + b, m);
    atomicMax(mo + b, o);
  }
}

static void absmax_into(const double2* X, long long per, int nw, unsigned* mx, cudaStream_t s) {
  int blocks = (int)std::min<long long>((per + 255) / 256, 128);
  k_absmax<<<dim3(blocks, nw), 256, 0, s>>>(X, per, per, mx);
}

// ---------------------------------------------------------------------------
// Per-step tables of the mixed path (coefficients frozen over the step).

// Toeplitz exchange planes T_n[t][t'] = vs_n(|t - t'|) (t != t'), real; and the
// FP32 copy of vs for the direct terms.
__global__ void k_toeplitz_planes(const WireDev* wires, const double* vs, const int* e,
                                  tc::PlaneSet dst, int nw, float* vsf) {
  // block (32, 8) over a 32 x 32 tile (rows t, columns t')
  __shared__ __align__(16) __half hs[2][32][40];
  const int b = blockIdx.z / 3, n = blockIdx.z % 3;
  const WireDev W = wires[b];
  const int nk = W.nk;
  const int t0 = blockIdx.y * 32, c0 = blockIdx.x * 32, tx = threadIdx.x;
  if (t0 >= nk || c0 >= nk) return;
  __shared__ __half th[2][64];   // hi, lo of the tile's 63 diagonals t - t' - (t0 - c0) + 31
  const int eb = e[b];
  const double* v = vs + 3 * W.off_vec + n * nk;
  const int tp = c0 + tx;
  const int tid = threadIdx.y * 32 + tx;
  if (tid < 63) {
    const int dd = tid - 31 + t0 - c0, d = dd < 0 ? -dd : dd;
    const float f = (d == 0 || d >= nk) ? 0.f : f64_to_f32(v[d], eb);
    const __half hi = __float2half_rn(f);
    th[0][tid] = hi;
    th[1][tid] = __float2half_rn(f - __half2float(hi));
  }
  if (t0 == 0 && threadIdx.y == 0 && tp < nk)
    vsf[((long long)b * 3 + n) * nk + tp] = f64_to_f32(v[tp]);
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = threadIdx.y + 8 * k;
    const bool in = t0 + i < nk && tp < nk;
    const int j = i - tx + 31;
    hs[0][i][tx] = in ? th[0][j] : __float2half_rn(0.f);
    hs[1][i][tx] = in ? th[1][j] : __float2half_rn(0.f);
  }
  __syncthreads();
  store_tiles(hs, 2, dst, n, b, t0, c0 >> 5, threadIdx.y * 32 + tx, 32 * blockDim.y);
}

__global__ void k_vs_max(const WireDev* wires, const double* vs, unsigned* mx) {
  const WireDev W = wires[blockIdx.x];
  unsigned long long m = 0;
  for (int i = threadIdx.x; i < 3 * W.nk; i += blockDim.x) m = max(m, absbits(vs[3 * W.off_vec + i]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx + blockIdx.x, bits_to_fmax(m));
}

// hbar A and hbar B in FP32 (dephasing.py:714-743 contraction matrices A[k][j] =
// Dh[j - k][k], B[k][j] = De[j - k][k], j != k) and max(2 hbar |A|, 2 hbar |B|).
// The block's sources Dh[q][k], q = j - k + Nk in a 63-wide band, k in its 32
// rows, are read row by row (coalesced) into shared memory.
__global__ void k_hab(const WireDev* wires, const double* De, const double* Dh, float* habf,
                      long long tot_mat, unsigned* mx) {
  __shared__ double ta[63][33], tb[63][33];
  const WireDev W = wires[blockIdx.z];
  const int nk = W.nk;
  const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int qbase = j0 - k0 - 31 + nk;
  const bool on_w = (W.flags & SBE_F_OFFDIAGDPH) != 0;
  {
    // block (32, 8): eight rows per thread, all loads issued before the stores
    double va[8], vb[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int qq = threadIdx.y + 8 * i, q = qbase + qq, k = k0 + threadIdx.x;
      const bool ok = on_w && qq < 63 && q >= 0 && q <= 2 * nk && k < nk;
      const long long di = W.off_dd + (long long)q * nk + k;
      va[i] = ok ? Dh[di] : 0.0;
      vb[i] = ok ? De[di] : 0.0;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int qq = threadIdx.y + 8 * i;
      if (qq < 63) {
        ta[qq][threadIdx.x] = va[i];
        tb[qq][threadIdx.x] = vb[i];
      }
    }
  }
  __syncthreads();
  const float hb = (float)kHbar;
  float m = 0.f;
  const int j = j0 + threadIdx.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int kk = threadIdx.y + 8 * i;
    const int k = k0 + kk;
    if (k >= nk || j >= nk) continue;
    const int qq = (j - k) - (j0 - k0) + 31;
    const float ha = (j != k) ? hb * f64_to_f32(ta[qq][kk]) : 0.f;
    const float hh = (j != k) ? hb * f64_to_f32(tb[qq][kk]) : 0.f;
    const long long o = W.off_mat + (long long)k * nk + j;
    habf[o] = ha;
    habf[tot_mat + o] = hh;
    m = fmaxf(m, 2.f * fmaxf(fabsf(ha), fabsf(hh)));
  }
  // one atomic per block (same-address atomics serialise)
  __shared__ float red[8];
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if (threadIdx.x == 0) red[threadIdx.y] = m;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int w = 1; w < 8; ++w) m = fmaxf(m, red[w]);
    atomicMax(mx + blockIdx.z, __float_as_uint(m));
  }
}

// Per-step weights of CalcGammaE/H (dephasing.py:29-103) per q: (pi/hbar) V^2 |x|
// with V = Vxx2 at iq[q]: [0] vee^2 |xe|, [1] veh^2 |xh|, [2] vhh^2 |xh|, [3] veh^2 |xe|.
__global__ void k_gamma_tab(const WireDev* wires, const double* vs, const int* iq,
                            const double* xeh, float* gtab, int nw) {
  const WireDev W = wires[blockIdx.y];
  const int nk = W.nk, b = blockIdx.y;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nk) return;
  const double* v = vs + 3 * W.off_vec;
  const int i = iq[W.off_vec + q];
  const double pih = kPi / kHbar;
  const double veh = v[i], vee = v[nk + i], vhh = v[2 * nk + i];
  const double xe = fabs(xeh[2 * W.off_vec + q]), xh = fabs(xeh[2 * W.off_vec + nk + q]);
  const long long o = (long long)b * nk + q, st = (long long)nw * nk;
  gtab[o] = f64_to_f32(pih * vee * vee * xe);
  gtab[st + o] = f64_to_f32(pih * veh * veh * xh);
  gtab[2 * st + o] = f64_to_f32(pih * vhh * vhh * xh);
  gtab[3 * st + o] = f64_to_f32(pih * veh * veh * xe);
}

// CalcGammaE/H in FP32 (same sums and index maps as k_gamma); one warp per (wire,
// k), lanes over q; occupations (real parts) staged in shared memory.
__global__ void k_gamma_f(const WireDev* wires, const double2* ne, const double2* nh,
                          const int* maps, const float* gtab, float* gamf, int nw) {
  extern __shared__ float occ[];
  const WireDev W = wires[blockIdx.y];
  const int nk = W.nk, b = blockIdx.y;
  float* pe = occ;
  float* ph = occ + nk;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    pe[i] = f64_to_f32(ne[W.off_vec + i].x);
    ph[i] = f64_to_f32(nh[W.off_vec + i].x);
  }
  __syncthreads();
  const int k = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (k >= nk) return;
  const long long vo = (long long)b * nk, st1 = (long long)nw * nk;
  if (!(W.flags & SBE_F_DIAGDPH)) {
    if (lane == 0) {
      gamf[vo + k] = (float)W.gam_e;
      gamf[st1 + vo + k] = (float)W.gam_h;
    }
    return;
  }
  const long long st = (long long)nk * nk;
  const int* m = maps + 6 * W.off_mat + (long long)k * nk;
  const float* g0 = gtab + vo;
  const float* g1 = gtab + st1 + vo;
  const float* g2 = gtab + 2 * st1 + vo;
  const float* g3 = gtab + 3 * st1 + vo;
  float ge = 0.f, gh = 0.f;
  for (int q = lane; q < nk; q += 32) {
    const int i0 = m[q], i1 = m[st + q], i2 = m[2 * st + q], i3 = m[3 * st + q];
    const int i4 = m[4 * st + q], i5 = m[5 * st + q];
    const bool k0ok = i0 >= 0 && i0 < nk;
    if (k0ok) {
      const float a = pe[i0], bb = ph[i0];
      ge += g0[q] * (a * (1.f - a));
      gh += g2[q] * (bb * (1.f - bb));
    }
    const bool ok1 = i1 >= 0 && i1 < nk, ok2 = i2 >= 0 && i2 < nk, ok3 = i3 >= 0 && i3 < nk;
    const bool ok4 = i4 >= 0 && i4 < nk, ok5 = i5 >= 0 && i5 < nk;
    if (ok3 && ok2 && ok1) {
      const float n1 = ph[i3], n2 = ph[i2], n3 = pe[i1];
      ge += g1[q] * (n1 * (1.f - n2) * n3 + (1.f - n1) * n2 * (1.f - n3));
    }
    if (ok5 && ok4 && ok1) {
      const float e1 = pe[i5], e2 = pe[i4], h3 = ph[i1];
      gh += g3[q] * (e1 * (1.f - e2) * h3 + (1.f - e1) * e2 * (1.f - h3));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    ge += __shfl_down_sync(0xffffffffu, ge, o);
    gh += __shfl_down_sync(0xffffffffu, gh, o);
  }
  if (lane == 0) {
    gamf[vo + k] = ge;
    gamf[st1 + vo + k] = gh;
  }
}

// Per-step phonon coupling per |k - k'| (phonons.py:140-268): Vep(d) = VC_ee(d) /
// E1D(d) Vscale and Vhp for holes, scaled by 2^-sP to pair with the FP32 tables.
__global__ void k_phon_tab(const WireDev* wires, const double* vs, const double* eps,
                           const int* sP, float* phf, int nw) {
  const WireDev W = wires[blockIdx.y];
  const int nk = W.nk, b = blockIdx.y;
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nk) return;
  const double* v = vs + 3 * W.off_vec;
  const double ep = eps[W.off_vec + d];
  phf[(long long)b * nk + d] = f64_to_f32(v[nk + d] / ep * W.vscale, -sP[b]);
  phf[((long long)nw + b) * nk + d] = f64_to_f32(v[2 * nk + d] / ep * W.vscale, -sP[b]);
}

// MBPE / MBPH (phonons.py:157-268) in FP32 from the scaled tables: Win, Wout of
// electrons and holes at the occupations in ne, nh (real parts) into wrate (FP64).
__global__ void k_phonon_rates_f(const WireDev* wires, const double2* nev, const double2* nhv,
                                 const float* phf, const float* epf, const float* eptf,
                                 const float* hpf, const float* hptf, double* wrate, int nw) {
  extern __shared__ float occ[];
  const WireDev W = wires[blockIdx.y];
  const int nk = W.nk, b = blockIdx.y, k = blockIdx.x;
  if (!(W.flags & SBE_F_PHONON)) {
    // no phonon rates: the carrier-carrier rates (EHs) are added to zeros
    if (threadIdx.x < 4) wrate[4 * W.off_vec + threadIdx.x * nk + k] = 0.0;
    return;
  }
  float* pe = occ;
  float* ph = occ + nk;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    pe[i] = f64_to_f32(nev[W.off_vec + i].x);
    ph[i] = f64_to_f32(nhv[W.off_vec + i].x);
  }
  __syncthreads();
  const float* ve = phf + (long long)b * nk;
  const float* vh = phf + ((long long)nw + b) * nk;
  const long long row = W.off_mat + (long long)k * nk;
  float wie = 0.f, woe = 0.f, wih = 0.f, woh = 0.f;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    const float a = pe[i], c = ph[i];
    if (k >= i) {
      const float v = ve[k - i];
      wie += v * a * epf[row + i];
      woe += v * (1.f - a) * eptf[row + i];
    }
    if (i >= k) {
      const float v = vh[i - k];
      wih += v * c * hpf[row + i];
      woh += v * (1.f - c) * hptf[row + i];
    }
  }
  __shared__ float red[4][4];
  float vals[4] = {wie, woe, wih, woh};
  for (int j = 0; j < 4; ++j)
    for (int o = 16; o > 0; o >>= 1) vals[j] += __shfl_down_sync(0xffffffffu, vals[j], o);
  if ((threadIdx.x & 31) == 0)
    for (int j = 0; j < 4; ++j) red[j][threadIdx.x >> 5] = vals[j];
  __syncthreads();
  if (threadIdx.x < 4) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
    wrate[4 * W.off_vec + threadIdx.x * nk + k] = f32_to_f64(t);
  }
}

// max(|re|, |im|) of the diagonals of C and D into mx[b] (after the relaxation
// step has rewritten them)
__global__ void k_diag_max(const WireDev* wires, const double2* C, const double2* D,
                           unsigned* mx) {
  const WireDev W = wires[blockIdx.x];
  unsigned long long m = 0;
  for (int k = threadIdx.x; k < W.nk; k += blockDim.x) {
    const long long o = W.off_mat + (long long)k * W.nk + k;
    const double2 a = C[o], d = D[o];
    m = max(m, max(max(absbits(a.x), absbits(a.y)), max(absbits(d.x), absbits(d.y))));
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx + blockIdx.x, bits_to_fmax(m));
}

// QWPolarization3 / QWRho5 reduction (qwoptics.py:809-1071) from the FP32 source
// GEMM outputs G[k][r] = sum_k' X[k][k'] e^{i k' r}: sums over k in FP32, the
// physical prefactors in FP64 per r.  Block (32 r) x (8 k-groups): thread (x, y)
// sums k = y, y + 8, ... of point r, the eight partial sums meet in shared memory.
__global__ void k_src_reduce_f(const WireDev* wires, const float2* ekrf, const float2* G,
                               long long tot_kr, const double* win, double2* src) {
  __shared__ float part[6][8][33];
  const WireDev W = wires[blockIdx.y];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int r = blockIdx.x * 32 + tx;
  const int nk = W.nk, nr = W.nr;
  float sx = 0.f, sy = 0.f, ser = 0.f, sei = 0.f, shr = 0.f, shi = 0.f;
  if (r < nr) {
    const float2* E = ekrf + W.off_kr;
    const float2* Gp = G + W.off_kr;
    const float2* Gc = G + tot_kr + W.off_kr;
    const float2* Gd = G + 2 * tot_kr + W.off_kr;
    // rows k = ty + 8 i in batches of four, all loads of a batch issued before
    // the sums (same order of the sums as one row at a time)
    for (int k0 = ty; k0 < nk; k0 += 32) {
      float2 e[4], gp[4], gc[4], gd[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + 8 * u;
        const long long o = (long long)(k < nk ? k : 0) * nr + r;
        e[u] = E[o];             // conj taken below
        gp[u] = Gp[o];
        gc[u] = Gc[o];
        gd[u] = Gd[o];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + 8 * u;
        if (k >= nk) break;
        const float re_part = e[u].x * gp[u].x + e[u].y * gp[u].y;
        sx += (k & 1) ? -re_part : re_part;
        sy += re_part;
        ser += e[u].x * gc[u].x + e[u].y * gc[u].y;
        sei += e[u].x * gc[u].y - e[u].y * gc[u].x;
        shr += e[u].x * gd[u].x + e[u].y * gd[u].y;
        shi += e[u].x * gd[u].y - e[u].y * gd[u].x;
      }
    }
  }
  part[0][ty][tx] = sx;
  part[1][ty][tx] = sy;
  part[2][ty][tx] = ser;
  part[3][ty][tx] = sei;
  part[4][ty][tx] = shr;
  part[5][ty][tx] = shi;
  __syncthreads();
  if (ty != 0 || r >= nr) return;
  float v[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    float a = 0.f;
#pragma unroll
    for (int g = 0; g < 8; ++g) a += part[i][g][tx];
    v[i] = a;
  }
  const double w = win[W.off_r + r];
  double2* out = src + 5 * W.off_r;
  const bool optics = (W.flags & SBE_F_OPTICS) != 0;
  const double pf = 2 * W.ehint / W.area / W.L;
  const double px = optics ? (W.dcv * f32_to_f64(v[0])) * w : 0.0;
  const double py = optics ? (W.dcv * f32_to_f64(v[1])) * w * W.yw : 0.0;
  const double pz = optics ? (-W.dcv * f32_to_f64(v[1])) * w * W.zsign : 0.0;
  out[r] = make_double2(px * pf, 0.0);
  out[nr + r] = make_double2(py * pf, 0.0);
  out[2 * nr + r] = make_double2(pz * pf, 0.0);
  const double f = w / (2.0 * W.L);
  out[3 * nr + r] = make_double2(f32_to_f64(v[2]) * f, f32_to_f64(v[3]) * f);
  out[4 * nr + r] = make_double2(f32_to_f64(v[4]) * f, f32_to_f64(v[5]) * f);
}

// ---------------------------------------------------------------------------
// Per-stage kernels.

// Sheared state planes: row 2 dd + c (dd = d + Nk - 1, c = re / im), column t':
// S[2dd + c][t'] = component c of X[t' + d][t'] (zero outside the matrix).
// The exchange sum  H[t][t+d] = sum_t' V(|t - t'|) X[t' + d][t']  is then T S.
// A block writes dd in [dd0, dd0 + 32) x t' in [t0, t0 + 32); the source elements
// lie in rows t0 + dd0 - (Nk - 1) ... + 62 of columns t0 ... t0 + 31, which are
// read row by row (coalesced) into shared memory and then read along diagonals
// (row stride 32 float2: diagonal reads are free of bank conflicts).
// The grid covers only the band: blockIdx.y counts the dd blocks from
// shear_first_block(t0) on (the other blocks hold zeros, which the buffer keeps
// from its initialisation); blockIdx.z = matrix n (0 P, 1 C, 2 D) * Nw + wire;
// block (32, 8).
// For C and D the block also writes the sum of its 32 values of every diagonal
// (unscaled FP32, in the fixed order t' = ddl, ddl + 1, ... cyclically) to
// dpart[((b * 2 + n - 1) * ndd + dd) * gridDim.x + blockIdx.x]; the traces of the
// direct Coulomb terms are their sums over the blocks that exist.
__global__ void k_shear_tiles(int nk, int nw, int ndd, const float2* X0, const float2* X1,
                              const float2* X2, const int* e, tc::PlaneSet dst, float2* dpart) {
  __shared__ float2 tile[63][32];
  __shared__ __align__(16) __half hs[2][64][40];   // hi, lo of rows 2 dd0 .. 2 dd0 + 63
  const int n = blockIdx.z / nw, b = blockIdx.z % nw;
  const int t0 = blockIdx.x * 32;
  const int dd0 = (shear_first_block(nk, t0) + blockIdx.y) * 32;
  if (dd0 >= ndd || !shear_block_live(nk, t0, dd0)) return;
  const float2* X = (n == 0 ? X0 : n == 1 ? X1 : X2) + (long long)b * nk * nk;
  const int rbase = t0 + dd0 - (nk - 1);
  const int tx = threadIdx.x, ty = threadIdx.y;
  {
    // eight rows per thread, all loads issued before the stores
    const int c = t0 + tx;
    float2 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int rr = ty + 8 * k, r = rbase + rr;
      const bool ok = rr < 63 && r >= 0 && r < nk && c < nk;
      v[k] = ok ? X[(long long)r * nk + c] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (ty + 8 * k < 63) tile[ty + 8 * k][tx] = v[k];
  }
  __syncthreads();
  if (n > 0 && ty == 0) {
    // diagonal partials: lane ddl starts at t' = ddl, so that the 32 lanes read
    // 32 different banks pairs at every step
    float sr = 0.f, si = 0.f;
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const int t = (tx + i) & 31;
      const float2 v = tile[t + tx][t];
      sr += v.x;
      si += v.y;
    }
    dpart[(((long long)b * 2 + n - 1) * ndd + dd0 + tx) * gridDim.x + blockIdx.x] =
        make_float2(sr, si);
  }
  const int eb = e[b];
#pragma unroll
  for (int kd = 0; kd < 4; ++kd) {
    const int ddl = ty + 8 * kd;
    // element (dd0 + ddl, t0 + tx) of the shear: source row rbase + tx + ddl (the
    // tile is zero outside the band and the matrix)
    const float2 t = tile[tx + ddl][tx];
    const float2 v = make_float2(f32_ldexp(t.x, eb), f32_ldexp(t.y, eb));
    const __half2 hi = __float22half2_rn(v);
    const float2 hf = __half22float2(hi);
    const __half2 lo = __float22half2_rn(make_float2(v.x - hf.x, v.y - hf.y));
    hs[0][2 * ddl][tx] = __low2half(hi);
    hs[1][2 * ddl][tx] = __low2half(lo);
    hs[0][2 * ddl + 1][tx] = __high2half(hi);
    hs[1][2 * ddl + 1][tx] = __high2half(lo);
  }
  __syncthreads();
  // 2 planes x 64 rows x 4 chunks of 16 bytes: two per thread; the rows of a plane
  // are contiguous in K-block t0 / 32
  const int tid = ty * 32 + tx;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int t = tid + 256 * u;
    const int pl = t >> 8, rr = (t >> 2) & 63, j = t & 3;
    const uint4 v = *reinterpret_cast<const uint4*>(&hs[pl][rr][8 * j]);
    *reinterpret_cast<uint4*>(dst.ptr + tc::chunk_elem(dst, n, pl, b, 2 * dd0 + rr, t0 >> 5, j)) =
        v;
  }
}

// The stage field in FP32.

__global__ void k_field_f(long long n, const double2* ek, const double2* dek, double frac,
                          float2* ekf) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 a = ek[i];
  if (dek) {
    // stage field Ek0 + frac dEk in FP64 (as the FP64 path's stage field)
    const double2 d = dek[i];
    a.x += frac * d.x;
    a.y += frac * d.y;
  }
  ekf[i] = f64_to_f32(a);
}

// H = Meh + diagonal energies + direct Coulomb terms + exchange sums
// (SBEs.py:1044-1131) in FP32: Heh, Hee' and Hhh' (diagonal removed) into hf.
// The exchange sums come from the FP32 GEMM output xsh[n][b][k1][k2] (the engine's
// epilogue un-shears the columns dd = k2 - k1 + Nk - 1 of the product).  The diagonal of
// Hee / Hhh (gap + kinetic energy) is formed in FP64 into dgE / dgH and split into
// FP32 hi / lo parts (dgf).  The block maximum of the operands goes to mx[b].
constexpr int HB_ROWS = 1;

__global__ void k_h_build(const WireDev* __restrict__ wires, const float2* __restrict__ ekf,
                          const float* __restrict__ vsf, const double* __restrict__ Ee,
                          const double* __restrict__ Eh, const float2* __restrict__ trf,
                          const float2* __restrict__ xsh, int have_x, float2* __restrict__ hf,
                          long long tot_mat, double2* __restrict__ dgE, double2* __restrict__ dgH,
                          float2* __restrict__ dgf, unsigned* __restrict__ mx) {
  const WireDev& W = wires[blockIdx.z];
  const int nk = W.nk, b = blockIdx.z, nw = gridDim.z;
  float hmax = 0.f;
  // HB_ROWS rows per block
  for (int rr = 0; rr < HB_ROWS; ++rr) {
  const int k1 = blockIdx.y * HB_ROWS + rr;
  for (int it = 0; it < 4; ++it) {
  const int k2 = blockIdx.x * blockDim.x * 4 + it * blockDim.x + threadIdx.x;
  if (k1 < nk && k2 < nk) {
    float2 heh = make_float2(0.f, 0.f), hee = heh, hhh = heh;
    if (W.flags & SBE_F_OPTICS) {
      int q = k1 - k2;
      if (q < 0) q += W.nr;
      const float2* ek = ekf + 3 * W.off_r;
      const float2 ex = ek[q], ey = ek[W.nr + q], ez = ek[2 * W.nr + q];
      const float sx = (k2 & 1) ? W.ed_x : -W.ed_x;       // -ehint Xcv
      const float sy = W.ed_y, sz = W.ed_z;
      heh.x = sx * ex.x + sy * ey.x + sz * ez.x;
      heh.y = sx * ex.y + sy * ey.y + sz * ez.y;
    }
    const bool exc = (W.flags & SBE_F_EXCITONS) != 0, lf = (W.flags & SBE_F_LF) != 0;
    const int d = k1 - k2;
    if (exc && lf && d != 0) {
      const float* v = vsf + (long long)b * 3 * nk;
      const float2* t = trf + (long long)b * 4 * nk;
      const int ad = d < 0 ? -d : d;
      const float v0 = v[ad], v1 = v[nk + ad], v2 = v[2 * nk + ad];
      const float2 trC = t[d + nk], trCm = t[-d + nk], trD = t[2 * nk + d + nk],
                   trDm = t[2 * nk - d + nk];
      hee.x = v1 * trC.x - v0 * trDm.x;
      hee.y = v1 * trC.y - v0 * trDm.y;
      hhh.x = v2 * trD.x - v0 * trCm.x;
      hhh.y = v2 * trD.y - v0 * trCm.y;
    }
    float2 xc = make_float2(0.f, 0.f), xd = xc;
    if (have_x) {
      const long long plane = (long long)nw * nk * nk;
      const long long xo = ((long long)b * nk + k1) * nk + k2;
      const float2 xe = xsh[xo];
      heh.x += xe.x;
      heh.y += xe.y;
      if (lf || d == 0) {
        xc = xsh[plane + xo];
        xd = xsh[2 * plane + xo];
      }
    }
    const long long o = W.off_mat + (long long)k1 * nk + k2;
    hf[o] = heh;
    if (d == 0) {
      // FP64 only on the diagonal (one element per row)
      const long long vo = (long long)b * nk + k1;
      const double2 ge = make_double2(Ee[W.off_vec + k1] + W.gap - (double)xc.x, -(double)xc.y);
      const double2 gh = make_double2(Eh[W.off_vec + k1] - (double)xd.x, -(double)xd.y);
      dgE[vo] = ge;
      dgH[vo] = gh;
      const float2 geh = make_float2((float)ge.x, (float)ge.y), ghh = make_float2((float)gh.x, (float)gh.y);
      dgf[vo] = geh;
      dgf[(long long)nw * nk + vo] = make_float2((float)(ge.x - (double)geh.x), (float)(ge.y - (double)geh.y));
      dgf[2ll * nw * nk + vo] = ghh;
      dgf[3ll * nw * nk + vo] = make_float2((float)(gh.x - (double)ghh.x), (float)(gh.y - (double)ghh.y));
      hee = make_float2(0.f, 0.f);
      hhh = hee;
    } else {
      hee.x -= xc.x;
      hee.y -= xc.y;
      hhh.x -= xd.x;
      hhh.y -= xd.y;
    }
    hf[tot_mat + o] = hee;
    hf[2 * tot_mat + o] = hhh;
    hmax = fmaxf(hmax, fmaxf(fmaxf(fmaxf(fabsf(heh.x), fabsf(heh.y)),
                                   fmaxf(fabsf(hee.x), fabsf(hee.y))),
                             fmaxf(fabsf(hhh.x), fabsf(hhh.y))));
  }
  }
  }
  __shared__ float red[4];
  for (int o = 16; o > 0; o >>= 1) hmax = fmaxf(hmax, __shfl_down_sync(0xffffffffu, hmax, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = hmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) hmax = fmaxf(hmax, red[w]);
    atomicMax(mx + b, __float_as_uint(hmax));
  }
}

// Planes of Hee', Hhh' (slots M_EE, M_HH) and of Hee' + i hbar B, Hhh' + i hbar A
// (slots M_EEX, M_HHX) from the FP32 values.
__global__ void k_hplanes(const float2* hee, const float2* hhh, const float* hA, const float* hB,
                          int nk, const int* e, tc::PlaneSet dst, int nw) {
  // block (32, 8) over a 32 x 32 tile; each slot's planes go through shared memory
  __shared__ __align__(16) __half hs[4][32][40];
  const int b = blockIdx.z;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32, tx = threadIdx.x, ty = threadIdx.y;
  const long long mm = (long long)nk * nk;
  const int eb = e[b];
  float2 a[4], h[4];
  float aa[4], bb[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int r = r0 + ty + 8 * k, c = c0 + tx;
    const bool in = r < nk && c < nk;
    const long long o = (long long)b * mm + (long long)r * nk + c;
    a[k] = in ? hee[o] : make_float2(0.f, 0.f);
    h[k] = in ? hhh[o] : make_float2(0.f, 0.f);
    bb[k] = in ? hB[o] : 0.f;
    aa[k] = in ? hA[o] : 0.f;
  }
  const int slot[4] = {M_EE, M_HH, M_EEX, M_HHX};
  const int tid = ty * 32 + tx;
  for (int sl = 0; sl < 4; ++sl) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = ty + 8 * k;
      const float2 v = sl == 0 ? a[k]
                       : sl == 1 ? h[k]
                       : sl == 2 ? make_float2(a[k].x, a[k].y + bb[k])
                                 : make_float2(h[k].x, h[k].y + aa[k]);
      hilo4(make_float2(f32_ldexp(v.x, eb), f32_ldexp(v.y, eb)), &hs[0][i][tx], &hs[1][i][tx],
            &hs[2][i][tx], &hs[3][i][tx]);
    }
    __syncthreads();
    store_tiles(hs, 4, dst, slot[sl], b, r0, c0 >> 5, tid, 256);
    __syncthreads();
  }
}

// s + e = a + b exactly (Knuth's two-sum in round-to-nearest FP32).  The peeled
// diagonal energies enter as products with the state every stage; a rounded FP32
// energy sum would be the same rounding every step, i.e. a frequency bias whose phase
// error grows with the number of oscillation periods, so the sum is kept exact as an
// unevaluated pair and the products round independently.
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
  return make_float2(s, e);
}

// RK4 stage update fused into the element-wise RHS passes (k_rhs_p, k_antiherm):
// the stage derivative k of an element is used where it is formed.  The
// arithmetic is that of the RK4 of the mixed path: FP32 k and sums k1 + 2 k2 +
// 2 k3; stages 1-3 write the next stage state in FP32 (xf = fp32(X) + f k) and,
// for C and D, its real diagonal in FP64; stage 4 adds to the FP64 state.  The
// maxima of the written state (all elements in mx, off-diagonal ones in mo when
// peel) feed the next stage's exponents.  stage 0: no update (the RHS is stored).
// The step's scale (dt / 2 or dt for the stage states, dt / 6 for the final sum)
// enters as an unevaluated FP32 pair fh + fl: an FP32-rounded dt would be the same
// relative error every step, i.e. a slightly different time step whose phase error
// grows with the number of oscillation periods of the state.  A pair product is
// fmaf(hi, x, lo x): the small term first, then one rounding of x hi + lo x (rounding
// x hi first would lose the correction in most cases and leave the constant's error
// as a bias).
struct Rk4Ctl {
  int stage, peel;
  float fh, fl;
  double2* X;      // FP64 state of this matrix, all wires
  const float2* x0;  // FP32 copy of the step-start state (stages 1-3)
  float2* acc;     // RK4 sums
  float2* xf;      // next stage state (FP32); may alias the pass's stage-state input
  double* dg;      // FP64 diagonal of the next stage state (C, D) or nullptr
  unsigned* mx;
  unsigned* mo;
};

__device__ __forceinline__ unsigned rk4_update(const Rk4Ctl& r, long long i, float2 kv, bool diag,
                                               long long dgi) {
  if (r.stage < 4) {
    if (r.stage == 1) {
      r.acc[i] = kv;
    } else {
      const float2 a = r.acc[i];
      r.acc[i] = make_float2(a.x + 2.f * kv.x, a.y + 2.f * kv.y);
    }
    const float2 xs = r.x0[i];   // fp32 of the FP64 state, converted once per step
    const float2 fk = make_float2(fmaf(r.fh, kv.x, r.fl * kv.x), fmaf(r.fh, kv.y, r.fl * kv.y));
    const float2 v = make_float2(xs.x + fk.x, xs.y + fk.y);
    r.xf[i] = v;
    if (diag && r.dg) r.dg[dgi] = r.X[i].x + f32_to_f64(fk.x);
    return max(__float_as_uint(v.x) & 0x7FFFFFFFu, __float_as_uint(v.y) & 0x7FFFFFFFu);
  }
  const double2 x = r.X[i];
  const float2 a = r.acc[i];
  const float sx = a.x + kv.x, sy = a.y + kv.y;
  const double2 v = make_double2(x.x + f32_to_f64(fmaf(r.fh, sx, r.fl * sx)),
                                 x.y + f32_to_f64(fmaf(r.fh, sy, r.fl * sy)));
  r.X[i] = v;
  return bits_to_fmax(max(absbits(v.x), absbits(v.y)));
}

// block maxima of the written states -> one atomic per block (blockDim 256)
__device__ __forceinline__ void rk4_block_max(const Rk4Ctl& r, int b, unsigned m, unsigned mof) {
  __shared__ unsigned red[2][8];
  for (int off = 16; off > 0; off >>= 1) {
    m = max(m, __shfl_down_sync(0xffffffffu, m, off));
    mof = max(mof, __shfl_down_sync(0xffffffffu, mof, off));
  }
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if ((t & 31) == 0) {
    red[0][t >> 5] = m;
    red[1][t >> 5] = mof;
  }
  __syncthreads();
  if (t == 0) {
    for (int w = 1; w < 8; ++w) {
      m = max(m, red[0][w]);
      mof = max(mof, red[1][w]);
    }
    atomicMax(r.mx + b, m);
    atomicMax(r.mo + b, mof);
  }
}

// dC (dD) from W = C' Hee'^T + P^H Heh^T (V = D' Hhh'^T + conj(P) Heh), where C'
// (D') is C (D) without its diagonal c (d): for Hermitian C, Hee (D, Hhh) the four
// terms of dCdt (dDdt) are W - W^H plus the peeled diagonal's (c_i - c_j) Hee'[j][i],
//   dX[i][j] = (W[i][j] - conj(W[j][i]) + (c_i - c_j) H'[j][i] + (g[j] - g[i]) X[i][j])
//              / (i hbar)
// with g the peeled energy diagonal.  Near equilibrium c_i - c_j is small against
// c_i H' and is formed from the hi / lo FP32 parts of c (the hi parts of close
// occupations differ exactly), so it does not carry the GEMM's rounding.  The
// result is exactly anti-Hermitian, which keeps C and D Hermitian.  A block owns
// the tile pair (bi, bj), (bj, bi) with bi <= bj and reads each W and H' element
// once.  W arrives in FP32 from the GEMMs (the hi*lo + lo*hi products, to
// which the hi*hi launch adds its K parts in order); g[j] - g[i] comes from the hi /
// lo FP32 parts of g.
__global__ void __launch_bounds__(256) k_antiherm(
    int nk, const float2* __restrict__ W, const float2* __restrict__ Hp, const float2* X,
    const float2* __restrict__ ghi, const float2* __restrict__ glo, const float* __restrict__ chi,
    const float* __restrict__ clo, float2* out, Rk4Ctl rk) {
  // tb / hb: W and H' of the mirror tile (rows j0.., columns i0..); vt: results;
  // gv / cv: g (hi, lo) and c (hi, lo) at the tile's rows i0.. (0) and columns j0.. (1)
  __shared__ float2 tb[32][33], hb[32][33], vt[32][33];
  __shared__ float2 gv[2][2][32];
  __shared__ float cv[2][2][32];
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bi > bj) return;
  const int b = blockIdx.z, tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = bi * 32, j0 = bj * 32;
  const long long mb = (long long)b * nk * nk;
  if (ty < 2) {
    const int k = (ty == 0 ? i0 : j0) + tx;
    const long long v = (long long)b * nk + (k < nk ? k : 0);
    gv[ty][0][tx] = ghi[v];
    gv[ty][1][tx] = glo[v];
    cv[ty][0][tx] = chi[v];
    cv[ty][1][tx] = clo[v];
  }
  // the mirror tile: four rows per thread, loads issued together
  {
    float2 w[4], h[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int ib = j0 + ty + 8 * q, jb = i0 + tx;
      const bool ok = ib < nk && jb < nk;
      const long long ob = mb + (long long)(ok ? ib : 0) * nk + (ok ? jb : 0);
      w[q] = W[ob];
      h[q] = Hp[ob];
      if (!ok) w[q] = h[q] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      tb[ty + 8 * q][tx] = w[q];
      hb[ty + 8 * q][tx] = h[q];
    }
  }
  __syncthreads();
  // 1 / hbar as an FP32 pair: one FP32 constant is 1e-8 off, a fixed relative error
  // of every rotation frequency that adds up over a pulse
  const float ihh = (float)(1.0 / kHbar), ihl = (float)(1.0 / kHbar - (double)ihh);
  unsigned mxv = 0, mov = 0;
  // the tile (i0.., j0..): i <= j wherever it is written
  {
    float2 w[4], x[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = i0 + ty + 8 * q, j = j0 + tx;
      const bool ok = i < nk && j < nk;
      const long long oa = mb + (long long)(ok ? i : 0) * nk + (ok ? j : 0);
      w[q] = W[oa];
      x[q] = X[oa];
    }
    const float2 gjh = gv[1][0][tx], gjl = gv[1][1][tx];
    const float cjh = cv[1][0][tx], cjl = cv[1][1][tx];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = ty + 8 * q;
      const int i = i0 + r, j = j0 + tx;
      const float2 a = w[q];                         // W[i][j]
      const float2 bt = tb[tx][r];                   // W[j][i]
      const float2 hji = hb[tx][r];                  // H'[j][i]
      const float2 gih = gv[0][0][r], gil = gv[0][1][r];
      const float2 dh = two_sum(gjh.x, -gih.x);            // exact difference of the hi parts
      const float drl = dh.y + (gjl.x - gil.x);
      const float di = (gjh.y - gih.y) + (gjl.y - gil.y);
      const float dc = (cv[0][0][r] - cjh) + (cv[0][1][r] - cjl);
      const float re = (a.x - bt.x) + dc * hji.x +
                       fmaf(dh.x, x[q].x, fmaf(drl, x[q].x, -di * x[q].y));
      const float im = (a.y + bt.y) + dc * hji.y +
                       fmaf(dh.x, x[q].y, fmaf(drl, x[q].y, di * x[q].x));
      const float2 v = make_float2(fmaf(im, ihh, im * ihl), -fmaf(re, ihh, re * ihl));
      vt[r][tx] = v;
      if (i < nk && j < nk && (bi < bj || j >= i)) {
        const long long o = mb + (long long)i * nk + j;
        if (rk.stage == 0) {
          out[o] = v;
        } else {
          const unsigned a = rk4_update(rk, o, v, i == j, (long long)b * nk + i);
          mxv = max(mxv, a);
          if (!rk.peel || i != j) mov = max(mov, a);
        }
      }
    }
  }
  __syncthreads();
  // the mirror tile as the conjugate transpose: dX is Hermitian by construction
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = ty + 8 * q;
    const int i = j0 + r, j = i0 + tx;
    if (i >= nk || j >= nk) continue;
    if (bi < bj || i > j) {
      const float2 v = vt[tx][r];
      const long long o = mb + (long long)i * nk + j;
      if (rk.stage == 0) {
        out[o] = make_float2(v.x, -v.y);
      } else {
        const unsigned a = rk4_update(rk, o, make_float2(v.x, -v.y), false, 0);
        mxv = max(mxv, a);
        mov = max(mov, a);
      }
    }
  }
  if (rk.stage != 0) rk4_block_max(rk, b, mxv, mov);
}

// dP of a stage from the FP32 commutator sums G (the engine's scaled products with
// the off-diagonal C', D'), following dpdt (SBEs.py:1942-1965):
//   dP[kh][ke] = (G + (1 - c[ke] - d[kh]) Heh[ke][kh] + (hh[kh] + ee[ke]) P) / (i hbar)
//                - (GamE[ke] + GamH[kh]) P
// in FP32 from the FP32 stage state P.  The peeled
// occupations c, d enter through the Pauli-blocking factor of the driving term and
// the peeled energy diagonals ee, hh as hi + lo FP32 parts.  32 x 32 tiles; Heh^T
// goes through shared memory so that every global access runs along rows.
__global__ void __launch_bounds__(256) k_rhs_p(
    int nk, int nw, const float2* __restrict__ G, const float2* __restrict__ hehf,
    const float2* X, const float2* __restrict__ dgf, const float* __restrict__ gamf,
    const float* __restrict__ cdf, float2* out, Rk4Ctl rk) {
  __shared__ float2 ht[32][33];
  // per-row (kh = m0 + r) values: hh hi, lo; GamH; d hi, lo
  __shared__ float2 rg[2][32];
  __shared__ float rv[3][32];
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * 32, n0 = blockIdx.x * 32;
  const long long mb = (long long)b * nk * nk, vb = (long long)b * nk, vn = (long long)nw * nk;
  const int tx = threadIdx.x, ty = threadIdx.y;
  {
    float2 h[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int n = n0 + ty + 8 * q, m = m0 + tx;
      const bool ok = n < nk && m < nk;
      h[q] = hehf[mb + (long long)(ok ? n : 0) * nk + (ok ? m : 0)];
      if (!ok) h[q] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) ht[ty + 8 * q][tx] = h[q];
  }
  if (ty == 0) {
    const long long v = vb + (m0 + tx < nk ? m0 + tx : 0);
    rg[0][tx] = dgf[2 * vn + v];
    rg[1][tx] = dgf[3 * vn + v];
    rv[0][tx] = gamf[vn + v];
    rv[1][tx] = cdf[2 * vn + v];
    rv[2][tx] = cdf[3 * vn + v];
  }
  __syncthreads();
  const int n = n0 + tx;
  const bool on = n < nk;
  // 1 / hbar as an FP32 pair (the rotation frequency of P to FP32 precision)
  const float ihh = (float)(1.0 / kHbar), ihl = (float)(1.0 / kHbar - (double)ihh);
  unsigned mxv = 0, mov = 0;
  const long long vnn = vb + (on ? n : 0);
  const float2 eh = dgf[vnn], el = dgf[vn + vnn];
  const float gamE = gamf[vnn];
  const float chi = cdf[vnn], clo = cdf[vn + vnn];
  float2 g[4], x[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int m = m0 + ty + 8 * q;
    const bool ok = on && m < nk;
    const long long o = mb + (long long)(ok ? m : 0) * nk + (ok ? n : 0);
    g[q] = G[o];
    x[q] = X[o];
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = ty + 8 * q, m = m0 + r;
    if (!on || m >= nk) continue;
    const float2 h0 = ht[tx][r];   // Heh[ke = n][kh = m]
    const float pb = ((1.f - chi) - rv[1][r]) - (clo + rv[2][r]);
    const float ax = g[q].x + pb * h0.x, ay = g[q].y + pb * h0.y;
    const float2 gh = rg[0][r], gl = rg[1][r];
    const float2 sh = two_sum(gh.x, eh.x);                 // exact sum of the hi parts
    const float derl = sh.y + (gl.x + el.x), dei = (gh.y + eh.y) + (gl.y + el.y);
    const float ar = ax + fmaf(sh.x, x[q].x, fmaf(derl, x[q].x, -dei * x[q].y));
    const float ai = ay + fmaf(sh.x, x[q].y, fmaf(derl, x[q].y, dei * x[q].x));
    const float gam = gamE + rv[0][r];
    const float2 kv = make_float2(fmaf(ai, ihh, ai * ihl) - gam * x[q].x,
                                  -fmaf(ar, ihh, ar * ihl) - gam * x[q].y);
    const long long o = mb + (long long)m * nk + n;
    if (rk.stage == 0) {
      out[o] = kv;
    } else {
      const unsigned a = rk4_update(rk, o, kv, false, 0);
      mxv = max(mxv, a);
      mov = max(mov, a);
    }
  }
  if (rk.stage != 0) rk4_block_max(rk, b, mxv, mov);
}

__global__ void k_f32_to_f64(long long n, const float2* a, double2* out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = f32_to_f64(a[i]);
}

__global__ void k_add_int(int n, const int* a, const int* b, int* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}

static tc::GemmJob job(Mixed* m, const tc::PlaneSet& A, const tc::PlaneSet& B, int M, int N,
                       int K, int cplx, int nterms, const tc::Term* t, int kskip,
                       const tc::EpiArgs& e, int mode = tc::MODE_FULL, int xonly = 0,
                       int ksplit = 1) {
  tc::GemmJob j{};
  tc::GemmDesc& d = j.d;
  d.A = A;
  d.B = B;
  d.mode = mode;
  d.xonly = xonly;
  d.ksplit = ksplit;
  d.M = M;
  d.N = N;
  d.K = K;
  d.complex_mode = cplx;
  d.nterms = nterms;
  for (int i = 0; i < nterms; ++i) d.t[i] = t[i];
  d.batch = m->nw;
  d.kskip = kskip;
  d.nk_shear = m->nk;
  j.e = e;
  return j;
}

// Launch a job list (built bucket by bucket, largest Nk first, so that the longest
// tiles start first): consecutive jobs of one N tile share a persistent launch,
// tc::MAX_JOBS per launch.
int launch_jobs(const std::vector<tc::GemmJob>& jobs, cudaStream_t s) {
  for (size_t i = 0; i < jobs.size();) {
    size_t j = i + 1;
    while (j < jobs.size() && j - i < (size_t)tc::MAX_JOBS && jobs[j].d.bn == jobs[i].d.bn) ++j;
    const int rc = tc_gemm_launch(jobs.data() + i, (int)(j - i), s);
    if (rc) return rc;
    i = j;
  }
  return SBE_OK;
}

// The GEMM jobs of one kind for bucket m.  Exchange: T_n S_n (eh, ee, hh), real, the
// K range limited to the sheared band, un-sheared FP32 output.  Commutators (term
// lists follow dpdt, SBEs.py:1942-1965; dCdt and dDdt, SBEs.py:2309-2327 and
// 2607-2625, through their W - W^H form): dP, and the hi*lo + lo*hi products of W and
// V (xonly); their hi*hi products in K parts (hs) run in sequence per tile, with one
// accumulator per real product, which the epilogue adds in order to the cross terms
// (MODE_HH, kseq, kacc: W - W^H is a small difference of large products near
// equilibrium).  Sources: [P; C; conj D] E.
void bucket_jobs(SbeCtx* c, Mixed* m, int kind, std::vector<tc::GemmJob>& out) {
  MixedAll* A = all_of(c);
  const long long tm = c->tot_mat, mm = (long long)m->nk * m->nk;
  const int nk = m->nk;
  const size_t first = out.size();
  if (kind == JK_EXCH) {
    for (int n = 0; n < 3; ++n) {
      tc::Term t{n, n, 0, 0, 1};
      tc::EpiArgs e{};
      e.kind = tc::EPI_F32;
      e.outf = m->xsh + (long long)n * m->nw * 2 * mm;
      e.out_bstride = 2 * mm;
      e.ldo = 2 * nk;
      e.unshear = nk;
      e.escale = m->esx();
      e.err = A->err;
      out.push_back(job(m, m->tp, m->sp, nk, 4 * nk, nk, 0, 1, &t, 1, e));
    }
  } else if (kind == JK_FULL || kind == JK_HH) {
    const tc::Term tP[4] = {{M_HHX, M_PT, 0, 0, 1}, {M_D, M_EH, 1, 0, -1},
                            {M_P, M_EEX, 0, 0, 1}, {M_EHT, M_C, 0, 1, -1}};
    const tc::Term tC[2] = {{M_C, M_EE, 0, 0, 1}, {M_PT, M_EH, 1, 0, 1}};
    const tc::Term tD[2] = {{M_D, M_HH, 0, 0, 1}, {M_P, M_EHT, 1, 0, 1}};
    // G buffer (FP32 complex, tot_mat each, indexed like the packed state): [W, V, dP
    // sums]: the dP launch writes the cross terms of W and V, the hi*hi launch that
    // follows adds its K parts to them in order
    float2* wf = reinterpret_cast<float2*>(c->G);   // the buffer holds 12 tot_mat float2
    const int hs = m->hs;
    auto epi = [&](float2* o) {
      tc::EpiArgs e{};
      e.kind = tc::EPI_RAWF;
      e.outf2 = o + m->bm;
      e.out_bstride = mm;
      e.ks_stride = tm;
      e.escale = m->esc();
      e.err = A->err;
      return e;
    };
    if (kind == JK_FULL) {
      out.push_back(job(m, m->pl, m->pl, nk, nk, nk, 1, 4, tP, 0, epi(wf + G_DP * tm)));
      // the hi*lo + lo*hi products of W and V
      out.push_back(job(m, m->pl, m->pl, nk, nk, nk, 1, 2, tC, 0, epi(wf + G_W * tm),
                        tc::MODE_FULL, 1));
      out.push_back(job(m, m->pl, m->pl, nk, nk, nk, 1, 2, tD, 0, epi(wf + G_V * tm),
                        tc::MODE_FULL, 1));
    } else {
      // the K parts of a tile in sequence in one CTA, summed by its epilogue
      out.push_back(job(m, m->pl, m->pl, nk, nk, nk, 1, 2, tC, 0, epi(wf + G_W * tm), tc::MODE_HH,
                        0, hs));
      out.push_back(job(m, m->pl, m->pl, nk, nk, nk, 1, 2, tD, 0, epi(wf + G_V * tm), tc::MODE_HH,
                        0, hs));
      out[out.size() - 1].d.kseq = out[out.size() - 2].d.kseq = hs > 1 ? 1 : 0;
      out[out.size() - 1].d.kacc = out[out.size() - 2].d.kacc = 1;
    }
  } else {
    float2* gf = reinterpret_cast<float2*>(c->G);
    for (int j = 0; j < 3; ++j) {
      tc::Term t{2 * j, 0, j == 2 ? 1 : 0, 0, 1};
      tc::EpiArgs e{};
      e.kind = tc::EPI_RAWF;
      e.outf2 = gf + j * c->tot_kr + m->bkr;
      e.out_bstride = (long long)nk * m->nr;
      e.ldo = m->nr;
      e.escale = m->ess();
      e.err = A->err;
      out.push_back(job(m, m->pl, m->ep, nk, m->nr, nk, 1, 1, &t, 0, e));
    }
  }
  if (kind != JK_HH)
    for (size_t i = first; i < out.size(); ++i) out[i].d.bn = m->bn[kind];
}

// The jobs of one kind of every bucket, largest Nk first.
static std::vector<tc::GemmJob> all_jobs(SbeCtx* c, int kind) {
  MixedAll* A = all_of(c);
  std::vector<tc::GemmJob> jobs;
  for (int i = (int)A->b.size() - 1; i >= 0; --i) bucket_jobs(c, A->b[i], kind, jobs);
  return jobs;
}

static void exponents_from(Mixed* m, const unsigned* mx, int* e, cudaStream_t s) {
  k_exponents<<<(m->nw + 127) / 128, 128, 0, s>>>(m->nw, mx, e, nullptr, nullptr);
}

// Per-step set-up of the mixed path: the frozen preparation (screening, rates,
// dephasing matrices with the FP32 Lorentzian sums) and its FP32 tables.
static int mixed_prep(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s) {
  MixedAll* A = all_of(c);
  launch_prep_scalar(c, C, D, s);   // occupations, screening (FP64, O(Nk) per wire)
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    cudaMemsetAsync(m->mxH(), 0, sizeof(unsigned) * nw, s);
    k_vs_max<<<nw, 256, 0, s>>>(m->dw, c->vs, m->mxH());
    exponents_from(m, m->mxH(), m->eT(), s);
    k_toeplitz_planes<<<dim3((nk + 31) / 32, (nk + 31) / 32, 3 * nw), dim3(32, 8), 0, s>>>(
        m->dw, c->vs, m->eT(), m->tp, nw, m->vsf);
    k_gamma_tab<<<dim3((nk + 127) / 128, nw), 128, 0, s>>>(m->dw, c->vs, c->iq, c->xeh, m->gtab,
                                                           nw);
    k_gamma_f<<<dim3((nk + 7) / 8, nw), 256, sizeof(float) * 2 * nk, s>>>(
        m->dw, c->ne, c->nh, c->maps, m->gtab, m->gamf, nw);
    k_phon_tab<<<dim3((nk + 127) / 128, nw), 128, 0, s>>>(m->dw, c->vs, c->eps, m->sP, m->phf,
                                                          nw);
    cudaMemsetAsync(m->mxAB(), 0, sizeof(unsigned) * nw, s);
  }
  if (c->any_offdiag) {
    ProfScope ps(c, 3, s);
    launch_offdiag_D(c, -1, nullptr, true, s);
  }
  for (Mixed* m : A->b) {
    const int T = (m->nk + 31) / 32;
    k_hab<<<dim3(T, T, m->nw), dim3(32, 8), 0, s>>>(m->dw, c->De, c->Dh, A->habf, c->tot_mat,
                                                    m->mxAB());
  }
  return cuda_check(cudaGetLastError(), "mixed prep");
}

// Relaxation (phonon in/out rates of the new occupations, FP32 sums) and charge
// normalisation after the step (SBEs.py:5677-5702), then the state maximum.
static void mixed_relax(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek,
                        double dt, cudaStream_t s) {
  MixedAll* A = all_of(c);
  launch_extract_diag(c, C, D, s);
  for (Mixed* m : A->b)
    k_phonon_rates_f<<<dim3(m->nk, m->nw), 128, sizeof(float) * 2 * m->nk, s>>>(
        m->dw, c->ne, c->nh, m->phf, A->epf, A->eptf, A->hpf, A->hptf, c->wrate, m->nw);
  launch_mbc_rates(c, -1, s, false, true);
  launch_relax_only(c, P, C, D, Ek, dt, s);
  for (Mixed* m : A->b) k_diag_max<<<m->nw, 256, 0, s>>>(m->dw, C, D, m->mxS());
}

// Stage-1 state of the mixed path from the FP64 state: FP32 copies (the first
// three tot_mat blocks of the FP32 view of the context's stage buffer), the FP64
// diagonals of C and D, and the maxima the stage's exponents need.
static void mixed_state_in(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                           cudaStream_t s) {
  MixedAll* A = all_of(c);
  const long long tm = c->tot_mat;
  float2* xf = reinterpret_cast<float2*>(c->xs);
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    const long long mm = (long long)nk * nk, vn = (long long)nw * nk, o = m->bm;
    cudaMemsetAsync(m->mxS(), 0, sizeof(unsigned) * nw, s);
    cudaMemsetAsync(m->mxO(), 0, sizeof(unsigned) * nw, s);
    const int blocks = (int)std::min<long long>((mm + 255) / 256, 128);
    k_state_in<<<dim3(blocks, nw), 256, 0, s>>>(P + o, nk, 0, m->mxS(), m->mxO(), xf + o, nullptr);
    k_state_in<<<dim3(blocks, nw), 256, 0, s>>>(C + o, nk, 1, m->mxS(), m->mxO(), xf + tm + o,
                                                m->xdg);
    k_state_in<<<dim3(blocks, nw), 256, 0, s>>>(D + o, nk, 1, m->mxS(), m->mxO(),
                                                xf + 2 * tm + o, m->xdg + vn);
  }
}

// One RHS evaluation of the mixed path on the FP32 stage state xs (P, C, D at
// xs, xs + tot_mat, xs + 2 tot_mat; the FP64 diagonals of C and D in each bucket's
// xdg; the state maxima already in mxS, mxO) with the wire-k field Ek + frac dEk
// (dEk may be null).  With stage 1-4 the RK4 update of that stage is fused into the
// element-wise passes (X64: the FP64 states P, C, D; the next stage state goes to
// the FP32 stage buffer and its maxima to mxS, mxO); stage 0 stores the RHS in kf.
static int mixed_stage(SbeCtx* c, const float2* xs, const double2* Ek, const double2* dEk,
                       double frac, int stage, double dt, double2* const* X64, cudaStream_t s) {
  MixedAll* A = all_of(c);
  const long long tm = c->tot_mat;
  const int have_x = (c->wires[0].flags & SBE_F_EXCITONS) ? 1 : 0;
  // stage field in FP32 (all wires)
  k_field_f<<<(int)((3 * c->tot_r + 255) / 256), 256, 0, s>>>(3 * c->tot_r, Ek, dEk, frac, A->ekf);
  // state exponents and planes: P and P^T from one read; C and D need only their own
  // layout (C^T = conj C and D^T = conj D for the Hermitian C and D).  eS: full state
  // maximum (sheared exchange operands); eO: maximum over P and the off-diagonal C, D
  // (commutator operands; the diagonals of C and D are peeled off and applied exactly
  // in the element-wise passes)
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    const long long vn = (long long)nw * nk;
    const float2 *P = xs + m->bm, *C = xs + tm + m->bm, *D = xs + 2 * tm + m->bm;
    k_stage_exponents<<<(nw + 127) / 128, 128, 0, s>>>(nw, m->mxS(), m->mxO(), m->mxH(),
                                                       m->eS(), m->eO(), m->eT(), m->esx(),
                                                       stage > 0);
    const dim3 tb(32, 8), tg((nk + 31) / 32, (nk + 31) / 32, nw);
    k_planes_nt<float2><<<tg, tb, 0, s>>>(P, nk, m->eO(), m->pl, M_P, M_PT, nw);
    k_planes_nt<float2><<<tg, tb, 0, s>>>(C, nk, m->eO(), m->pl, M_C, -1, nw, m->cdf, m->xdg);
    k_planes_nt<float2><<<tg, tb, 0, s>>>(D, nk, m->eO(), m->pl, M_D, -1, nw, m->cdf + 2 * vn,
                                          m->xdg + vn);
    if (have_x) {
      // the traces of C and D (direct terms) come from the shear's diagonal partials
      const int nbk = (nk + 31) / 32, ndd = 32 * ((2 * nk + 31) / 32);
      int ny = 0;   // dd blocks of the band per t' block
      for (int i = 0; i < nbk; ++i) {
        int cnt = 0;
        for (int j = shear_first_block(nk, 32 * i); 32 * j < ndd; ++j)
          if (shear_block_live(nk, 32 * i, 32 * j)) cnt = j - shear_first_block(nk, 32 * i) + 1;
        ny = std::max(ny, cnt);
      }
      k_shear_tiles<<<dim3(nbk, ny, 3 * nw), dim3(32, 8), 0, s>>>(nk, nw, ndd, P, C, D, m->eS(),
                                                                 m->sp, m->tpart);
      k_trace_from_shear<<<dim3((2 * nk - 1 + 127) / 128, 2, nw), 128, 0, s>>>(nk, nbk, ndd,
                                                                               m->tpart, m->trf);
    }
  }
  int rc = SBE_OK;
  if (have_x) {
    // the three exchange products (eh, ee, hh) of every bucket
    ProfScope ps(c, 1, s);
    rc = launch_jobs(all_jobs(c, JK_EXCH), s);
    if (rc) return rc;
  }
  // the Hamiltonians: Meh + diagonal + direct + exchange, diagonal peeled; their planes
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    k_h_build<<<dim3((nk + 511) / 512, (nk + HB_ROWS - 1) / HB_ROWS, nw), 128, 0, s>>>(
        m->dw, A->ekf, m->vsf, c->Ee, c->Eh, m->trf, reinterpret_cast<const float2*>(m->xsh),
        have_x, A->hf, tm, m->dgE, m->dgH, m->dgf, m->mxH());
    // H exponent: max over the operands and the step's 2 hbar |A|, |B|
    k_exponents2_sum<<<(nw + 127) / 128, 128, 0, s>>>(nw, m->mxH(), m->mxAB(), m->eH(), m->eO(),
                                                      m->esc());
    const dim3 tb(32, 8), tg((nk + 31) / 32, (nk + 31) / 32, nw);
    k_planes_nt<float2><<<tg, tb, 0, s>>>(A->hf + m->bm, nk, m->eH(), m->pl, M_EH, M_EHT, nw);
    k_hplanes<<<tg, tb, 0, s>>>(A->hf + tm + m->bm, A->hf + 2 * tm + m->bm, A->habf + m->bm,
                                A->habf + tm + m->bm, nk, m->eH(), m->pl, nw);
  }
  // commutator GEMMs: dP and the cross terms of W and V, then the hi*hi products of
  // W and V (the partials of W and V meet in the anti-Hermitian pass)
  {
    ProfScope ps(c, 0, s);
    rc = launch_jobs(all_jobs(c, JK_FULL), s);
    if (rc) return rc;
  }
  {
    ProfScope ps(c, 0, s);
    rc = launch_jobs(all_jobs(c, JK_HH), s);
    if (rc) return rc;
  }
  float2* wf = reinterpret_cast<float2*>(c->G);
  // stage buffers (FP32, 3 tot_mat each): the step-start state, then the stage states
  float2* x0 = reinterpret_cast<float2*>(c->xs);
  float2* xn = x0 + 3 * tm;
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    const long long vn = (long long)nw * nk, o = m->bm;
    const float2 *P = xs + o, *C = xs + tm + o, *D = xs + 2 * tm + o;
    // this bucket's slices of the G buffer (see bucket_jobs)
    const float2* gp = wf + G_DP * tm;
    Rk4Ctl rk[3];
    for (int i = 0; i < 3; ++i) {
      rk[i] = Rk4Ctl{};
      rk[i].stage = stage;
      rk[i].peel = i > 0;
      // the stage scale as an exact FP32 pair (see Rk4Ctl)
      const double f = stage == 4 ? dt / 6.0 : (stage == 3 ? dt : 0.5 * dt);
      rk[i].fh = (float)f;
      rk[i].fl = (float)(f - (double)rk[i].fh);
      rk[i].X = X64 ? X64[i] + o : nullptr;
      rk[i].x0 = x0 + i * tm + o;
      rk[i].acc = A->accf + i * tm + o;
      rk[i].xf = xn + i * tm + o;
      rk[i].dg = i > 0 ? m->xdg + (i - 1) * vn : nullptr;
      rk[i].mx = m->mxS();
      rk[i].mo = m->mxO();
    }
    const dim3 ag((nk + 31) / 32, (nk + 31) / 32, nw), ab(32, 8);
    k_rhs_p<<<ag, ab, 0, s>>>(nk, nw, gp + o, A->hf + o, P, m->dgf, m->gamf, m->cdf, A->kf + o,
                              rk[0]);
    k_antiherm<<<ag, ab, 0, s>>>(nk, wf + G_W * tm + o, A->hf + tm + o, C, m->dgf,
                                 m->dgf + vn, m->cdf, m->cdf + vn, A->kf + tm + o, rk[1]);
    k_antiherm<<<ag, ab, 0, s>>>(nk, wf + G_V * tm + o, A->hf + 2 * tm + o, D,
                                 m->dgf + 2 * vn, m->dgf + 3 * vn, m->cdf + 2 * vn,
                                 m->cdf + 3 * vn, A->kf + 2 * tm + o, rk[2]);
  }
  return cuda_check(cudaGetLastError(), "mixed stage");
}

// Sources of the new state through the engine: G = [P; C; conj(D)] E (FP32
// outputs), then the per-r reductions.  mxS holds the state maximum when
// state_max_ready is set.
static int mixed_sources(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                         double2* src, int state_max_ready, cudaStream_t s) {
  MixedAll* A = all_of(c);
  for (Mixed* m : A->b) {
    const int nk = m->nk, nw = m->nw;
    const long long mm = (long long)nk * nk, o = m->bm;
    if (!state_max_ready) {
      cudaMemsetAsync(m->mxS(), 0, sizeof(unsigned) * nw, s);
      absmax_into(P + o, mm, nw, m->mxS(), s);
      absmax_into(C + o, mm, nw, m->mxS(), s);
      absmax_into(D + o, mm, nw, m->mxS(), s);
    }
    exponents_from(m, m->mxS(), m->eS(), s);
    const double2* st[3] = {P + o, C + o, D + o};
    const dim3 tb(32, 8), tg((nk + 31) / 32, (nk + 31) / 32, nw);
    for (int i = 0; i < 3; ++i)
      k_planes_nt<double2><<<tg, tb, 0, s>>>(st[i], nk, m->eS(), m->pl, 2 * i, -1, nw);
    k_add_int<<<(nw + 127) / 128, 128, 0, s>>>(nw, m->eS(), m->eE(), m->ess());
  }
  float2* gf = reinterpret_cast<float2*>(c->G);
  {
    ProfScope ps(c, 2, s);
    const int rc = launch_jobs(all_jobs(c, JK_SRC), s);
    if (rc) return rc;
  }
  for (Mixed* m : A->b)
    k_src_reduce_f<<<dim3((m->nr + 31) / 32, m->nw), dim3(32, 8), 0, s>>>(
        m->dw, A->ekrf, gf, c->tot_kr, c->window, src);
  launch_sources_final(c, c->ne, c->nh, src, s);
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
  MixedAll* A = all_of(c);
  const long long n = c->tot_mat;
  mixed_state_in(c, P, C, D, s);
  rc = mixed_stage(c, reinterpret_cast<const float2*>(c->xs), Ek, nullptr, 0.0, 0, 0.f, nullptr,
                   s);
  if (rc) return rc;
  const int g = (int)((n + 255) / 256);
  k_f32_to_f64<<<g, 256, 0, s>>>(n, A->kf, dP);
  k_f32_to_f64<<<g, 256, 0, s>>>(n, A->kf + n, dC);
  k_f32_to_f64<<<g, 256, 0, s>>>(n, A->kf + 2 * n, dD);
  return cuda_check(cudaGetLastError(), "rhs_mixed");
}

int rk4_mixed(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek0,
              const double2* dEk, double dt, double2* src, cudaStream_t s) {
  int rc = mixed_ensure(c, s);
  if (rc) return rc;
  rc = mixed_prep(c, C, D, s);
  if (rc) return rc;
  const long long n = c->tot_mat;
  const double frac[4] = {0.0, 0.5, 0.5, 1.0};
  // FP32 stage buffers in the FP64 stage-state block (6 tot_mat float2): the
  // step-start state (kept for the RK4 updates), then the stage states of stages 2-4
  float2* x0 = reinterpret_cast<float2*>(c->xs);
  mixed_state_in(c, P, C, D, s);
  double2* X64[3] = {P, C, D};
  for (int st = 1; st <= 4; ++st) {
    // the RHS of this stage (stage field Ek0 + frac dEk) and its RK4 update (fused
    // into the element-wise passes)
    rc = mixed_stage(c, st == 1 ? x0 : x0 + 3 * n, Ek0, dEk, frac[st - 1], st, dt, X64, s);
    if (rc) return rc;
  }
  mixed_relax(c, P, C, D, Ek0, dt, s);   // the new diagonals join the maximum
  // DC transport moves every element: the sources then measure the maximum themselves
  return mixed_sources(c, P, C, D, src, any_dc(c) ? 0 : 1, s);
}

}  // namespace sbe

using namespace sbe;

__global__ void k_convert_selftest(const double* din, const float* fin, long long n, float* fout,
                                   double* dout) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  fout[i] = f64_to_f32(din[i]);
  dout[i] = f32_to_f64(fin[i]);
}

// Diagnostic entry (no counterpart in the reference): the integer-pipe
// conversions of the mixed path, f_out = fp32(d_in) and d_out = fp64(f_in).
extern "C" int sbe_convert_selftest(const double* d_in, const float* f_in, long long n,
                                    float* f_out, double* d_out, void* stream) {
  if (!d_in || !f_in || !f_out || !d_out || n < 0)
    return fail(SBE_ERR_ARG, "sbe_convert_selftest: bad arguments");
  if (n == 0) return SBE_OK;
  k_convert_selftest<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(d_in, f_in, n,
                                                                               f_out, d_out);
  return cuda_check(cudaGetLastError(), "sbe_convert_selftest");
}

// Device-side error flag of the engine (bounded waits that gave up), read and
// cleared after the stream has drained.
extern "C" int sbe_ctx_check(SbeCtx* c, void* stream) {
  if (!c) return fail(SBE_ERR_ARG, "sbe_ctx_check: null context");
  int rc = cuda_check(cudaStreamSynchronize(as_stream(stream)), "sbe_ctx_check");
  if (rc) return rc;
  MixedAll* A = all_of(c);
  if (!A) return SBE_OK;
  int h = 0;
  rc = cuda_check(cudaMemcpy(&h, A->err, sizeof(int), cudaMemcpyDeviceToHost),
                  "sbe_ctx_check: read flag");
  if (rc) return rc;
  if (h) {
    cudaMemset(A->err, 0, sizeof(int));
    return fail(SBE_ERR_TIMEOUT, "a tensor-core pipeline wait timed out (results of the "
                                 "affected calls are invalid)");
  }
  return SBE_OK;
}

extern "C" int sbe_wait_selftest(SbeCtx* c, int* gave_up, void* stream) {
  if (!c || !gave_up) return fail(SBE_ERR_ARG, "sbe_wait_selftest: null argument");
  MixedAll* A = all_of(c);
  if (!A)
    return fail(SBE_ERR_ARG, "sbe_wait_selftest: no mixed-precision workspace yet (make a "
                             "mixed-precision call first)");
  cudaStream_t s = as_stream(stream);
  int* d = nullptr;
  if (cudaMallocAsync(&d, sizeof(int), s) != cudaSuccess)
    return fail(SBE_ERR_OOM, "sbe_wait_selftest: scratch allocation failed");
  int rc = tc_wait_selftest(A->err, d, s);
  int h = 0;
  if (!rc)
    rc = cuda_check(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s),
                    "sbe_wait_selftest: read result");
  cudaFreeAsync(d, s);
  if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "sbe_wait_selftest");
  *gave_up = h;
  return rc;
}

extern "C" int sbe_tc_selftest(int nk, int nbatch, const double* A, const double* B, int opA,
                               int opB, int complex_mode, double* out, void* stream) {
  if (nk < 8 || nk % 8 || nbatch < 1 || !A || !B || !out || opA < 0 || opA > 3 || opB < 0 ||
      opB > 3)
    return fail(SBE_ERR_ARG, "sbe_tc_selftest: bad arguments (nk must be a multiple of 8)");
  cudaStream_t s = as_stream(stream);
  const int npl = complex_mode ? 4 : 2;
  const long long mm = (long long)nk * nk;
  tc::PlaneSet ps = tc::make_planeset(nullptr, 2, npl, nbatch, nk, nk);
  int* ints = nullptr;
  unsigned* mx = nullptr;
  const size_t pbytes = tc::planeset_bytes(ps);
  if (cudaMallocAsync(&ps.ptr, pbytes, s) != cudaSuccess ||
      cudaMallocAsync(&ints, sizeof(int) * (3 * nbatch + 1), s) != cudaSuccess ||
      cudaMallocAsync(&mx, sizeof(unsigned) * nbatch, s) != cudaSuccess)
    return fail(SBE_ERR_OOM, "sbe_tc_selftest: scratch");
  cudaMemsetAsync(ps.ptr, 0, pbytes, s);
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
  launch_planes(a2, mm, nk, nbatch, tA, eA, ps, 0, !complex_mode, s);
  launch_planes(b2, mm, nk, nbatch, tB, eB, ps, 1, !complex_mode, s);
  int rc = SBE_OK;
  tc::GemmDesc d{};
  d.M = d.N = d.K = nk;
  d.complex_mode = complex_mode ? 1 : 0;
  d.nterms = 1;
  d.t[0] = tc::Term{0, 1, cA, cB, 1};
  d.batch = nbatch;
  d.A = ps;
  d.B = ps;
  tc::EpiArgs e{};
  e.kind = tc::EPI_RAW;
  e.out = (double2*)out;
  e.out_bstride = mm;
  e.escale = es;
  e.err = err;
  rc = tc_gemm_launch(d, e, s);
  if (rc) return rc;
  int herr = 0;
  cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  rc = cuda_check(cudaStreamSynchronize(s), "sbe_tc_selftest");
  cudaFreeAsync(ps.ptr, s);
  cudaFreeAsync(ints, s);
  cudaFreeAsync(mx, s);
  if (rc) return rc;
  if (herr) return fail(SBE_ERR_TIMEOUT, "sbe_tc_selftest: a pipeline wait timed out");
  return SBE_OK;
}
