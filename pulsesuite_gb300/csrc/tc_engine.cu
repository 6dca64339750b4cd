// tcgen05 / TMA / TMEM split-precision GEMM engine (see tc_gemm.cuh).
#include <cudaTypedefs.h>

#include "sbe_ctx.cuh"
#include "fp_bits.cuh"
#include "tc_gemm.cuh"

namespace sbe {
namespace tc {

// ---------------------------------------------------------------------------
// PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after ~2 s of clock cycles (or when another role
// already gave up), records the failure and returns false.
constexpr long long TIMEOUT_CYCLES = 4000000000ll;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err,
                                          volatile int* local_abort) {
  if (mbar_try_wait(bar, parity)) return true;
  long long t0 = clock64();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*local_abort) return false;
    if (clock64() - t0 > TIMEOUT_CYCLES) {
      atomicExch(err, 1);
      *local_abort = 1;
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2, int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4),
      "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// K-major operand in shared memory with 64-byte rows and the 64B swizzle (the
// layout TMA SWIZZLE_64B writes): 8-row groups are 512 bytes apart.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);  // start address (16-byte units)
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused when swizzled)
  d |= (uint64_t)(512 >> 4) << 32;          // stride byte offset: 8 rows x 64 B
  d |= (uint64_t)1 << 46;                   // descriptor version for tcgen05
  d |= (uint64_t)4 << 61;                   // swizzle mode: 64B
  return d;
}

// kind::f16 instruction descriptor: D = F32, A = B = F16, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, int negA) {
  return (1u << 4) | ((uint32_t)negA << 13) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// ---------------------------------------------------------------------------
// epilogues

__device__ __forceinline__ double2 cmuld(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One 16-column chunk of accumulators of row m (re[], im[]: FP32).
__device__ void epilogue_chunk(const GemmDesc& d, const EpiArgs& e, int b, int m, int n0,
                               const float* re, const float* im) {
  if (m >= d.M) return;
  const double sc = ldexp(1.0, -e.escale[b]);
  if (e.kind == EPI_F32) {
    float* o = e.outf + (long long)b * e.out_bstride + (long long)m * d.N + n0;
    const float scf = (float)sc;
    if (n0 + 16 <= d.N) {
      float4* o4 = reinterpret_cast<float4*>(o);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        o4[j] = make_float4(re[4 * j] * scf, re[4 * j + 1] * scf, re[4 * j + 2] * scf,
                            re[4 * j + 3] * scf);
    } else {
      for (int j = 0; j < 16 && n0 + j < d.N; ++j) o[j] = re[j] * scf;
    }
    return;
  }
  if (e.kind == EPI_RAW) {
    // exact widening and power-of-two scaling on the integer pipe
    double2* o = e.out + (long long)b * e.out_bstride + (long long)m * d.N;
    const int es = -e.escale[b];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      int n = n0 + j;
      if (n < d.N)
        o[n] = make_double2(f32_to_f64_scaled(re[j], es),
                            d.complex_mode ? f32_to_f64_scaled(im[j], es) : 0.0);
    }
    return;
  }
  if (e.kind == EPI_RAWF) {
    float2* o = e.outf2 + (long long)b * e.out_bstride + (long long)m * d.N;
    const int es = -e.escale[b];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      int n = n0 + j;
      if (n < d.N) o[n] = make_float2(f32_ldexp(re[j], es), f32_ldexp(im[j], es));
    }
    return;
  }
  if (e.kind == EPI_RHSF) {
    // dP[kh=m][ke=n] = (G + (hh[kh] + ee[ke]) P + (1 - c[ke] - d[kh]) Heh[ke][kh])
    //                 / (i hbar) - (gE+gH) P
    // in FP32 (the peeled diagonal energies add, so no cancellation), from the FP64
    // stage state P converted on the integer pipe.  G holds the products with the
    // off-diagonal C', D'; the peeled occupations c, d enter through the
    // Pauli-blocking factor of the driving term Heh^T - Heh^T diag(c) - (Heh diag(d))^T.
    const int nk = e.nk, nw = e.nw;
    const long long mb = (long long)b * nk * nk, vb = (long long)b * nk, vn = (long long)nw * nk;
    const float ih = (float)(1.0 / 1.0545718176461565e-34);
    const int es = -e.escale[b];
    const double2* X = e.X + mb + (long long)m * nk;
    const float2 gh = e.dgf[2 * vn + vb + m], gl = e.dgf[3 * vn + vb + m];
    const float gamH = e.gamf[vn + vb + m];
    const float dh = e.cdf[2 * vn + vb + m], dl = e.cdf[3 * vn + vb + m];
    float2* o = e.outf2 + mb + (long long)m * nk;
#pragma unroll 4
    for (int j = 0; j < 16; ++j) {
      const int n = n0 + j;
      if (n >= nk) break;
      const float gr = f32_ldexp(re[j], es), gi = f32_ldexp(im[j], es);
      const float2 x = f64_to_f32(X[n]);
      const float2 h0 = e.hehf[mb + (long long)n * nk + m];
      const float pb = ((1.f - e.cdf[vb + n]) - dh) - (e.cdf[vn + vb + n] + dl);
      const float2 h = make_float2(pb * h0.x, pb * h0.y);
      const float2 eh = e.dgf[vb + n], el = e.dgf[vn + vb + n];
      const float der = (gh.x + eh.x) + (gl.x + el.x), dei = (gh.y + eh.y) + (gl.y + el.y);
      const float ar = gr + (der * x.x - dei * x.y) + h.x;
      const float ai = gi + (der * x.y + dei * x.x) + h.y;
      const float gam = e.gamf[vb + n] + gamH;
      o[n] = make_float2(ai * ih - gam * x.x, -ar * ih - gam * x.y);
    }
    return;
  }
  if (e.kind == EPI_RHS) {
    // RHS of the state X: out = G/(i hbar) * sc + diagonal (peeled) terms, FP64.
    const int nk = e.nk;
    const long long mb = (long long)b * nk * nk;
    const double ih = 1.0 / 1.0545718176461565e-34;
    const double2* X = e.X + mb;
    const double2* gE = e.dgE + (long long)b * nk;
    const double2* gH = e.dgH + (long long)b * nk;
    double2* o = e.out + mb + (long long)m * nk;
#pragma unroll 4
    for (int j = 0; j < 16; ++j) {
      int n = n0 + j;
      if (n >= nk) break;
      double gr = re[j] * sc, gi = im[j] * sc;        // G = accumulated products (J)
      double2 x = X[(long long)m * nk + n];
      double2 v;
      if (e.which == 0) {
        // dP[kh=m][ke=n]: (G + (hh[kh] + ee[ke]) P + Heh[ke][kh])/(i hbar) - (gE+gH) P
        double2 h = e.Heh[mb + (long long)n * nk + m];
        double2 de = make_double2(gH[m].x + gE[n].x, gH[m].y + gE[n].y);
        double2 dx = cmuld(de, x);
        double ar = gr + dx.x + h.x, ai = gi + dx.y + h.y;
        double gam = e.gamE[(long long)b * nk + n] + e.gamH[(long long)b * nk + m];
        v = make_double2(ai * ih - gam * x.x, -ar * ih - gam * x.y);
      } else {
        const double2* g = (e.which == 1) ? gE : gH;
        double2 de = make_double2(g[n].x - g[m].x, g[n].y - g[m].y);   // (e[k2] - e[k1]) X
        double2 dx = cmuld(de, x);
        double ar = gr + dx.x, ai = gi + dx.y;
        v = make_double2(ai * ih, -ar * ih);
      }
      o[n] = v;
    }
    return;
  }
  if (e.kind == EPI_EXCH) {
    // exchange GEMM output: column n = 2*dd + c (dd = d + nk - 1, c = re/im) of
    // row t; H[t][t+d] gets the exchange sum X.  Real mode: only re[] used.
    const int nk = e.nk;
    double2* H = e.out + (long long)b * e.out_bstride;
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      int n = n0 + j;
      int dd = n >> 1;
      int dshift = dd - (nk - 1);
      int k2 = m + dshift;
      if (dd >= 2 * nk - 1 || k2 < 0 || k2 >= nk) continue;
      double xr = re[j] * sc, xi = re[j + 1] * sc;
      long long o = (long long)m * nk + k2;
      if (e.which == 0) {
        H[o] = make_double2(H[o].x + xr, H[o].y + xi);
      } else if (e.lf || dshift == 0) {
        H[o] = make_double2(H[o].x - xr, H[o].y - xi);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// the kernel

template <int BNT, bool SPLIT>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
              const GemmDesc d, const EpiArgs e) {
  constexpr int BTB = BNT * BK * 2;   // B tile bytes per plane
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int npl = d.complex_mode ? 4 : 2;
  const int stage_bytes = npl * (A_TILE_BYTES + BTB);
  const int nstage = (192 * 1024) / stage_bytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + nstage * stage_bytes);
  uint64_t* empty = full + 8;
  uint64_t* accb = empty + 8;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accb + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x & 31;
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BNT;
  const uint32_t ncols = d.complex_mode ? 512 : 256;

  // K range of this tile (the sheared exchange operand is zero outside it)
  int kb_begin = 0, kb_end = (d.K + BK - 1) / BK;
  if (d.kskip) {
    const int nk = d.nk_shear;
    int dd_lo = n0 / 2, dd_hi = min((n0 + BNT) / 2, 2 * nk - 1) - 1;
    int dlo = dd_lo - (nk - 1), dhi = dd_hi - (nk - 1);
    int tlo = max(0, -dhi), thi = min(nk - 1, nk - 1 - dlo);
    kb_begin = tlo / BK;
    kb_end = (thi >= tlo) ? thi / BK + 1 : kb_begin;
  }
  if (d.kb_hi > d.kb_lo) {
    kb_begin = d.kb_lo;
    kb_end = d.kb_hi;
  }
  const int nkb = kb_end - kb_begin;
  const int n_iters = d.nterms * nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < nstage; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accb, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, ncols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0 && n_iters > 0) {
    // ---------------- TMA producer ----------------
    for (int it = 0; it < n_iters; ++it) {
      const int s = it % nstage;
      const uint32_t ph = (uint32_t)((it / nstage) & 1);
      if (!mbar_wait(&empty[s], ph ^ 1u, e.err, abort_flag)) break;
      const Term T = d.t[it / nkb];
      const int kb = kb_begin + it % nkb;
      uint8_t* sa = smem + s * stage_bytes;
      uint8_t* sb = sa + npl * A_TILE_BYTES;
      mbar_expect_tx(&full[s], (uint32_t)stage_bytes);
      for (int p = 0; p < npl; ++p) {
        tma_load_5d(sa + p * A_TILE_BYTES, &ma, &full[s], kb * BK, m0, b, p, T.a_mat);
        tma_load_5d(sb + p * BTB, &mb, &full[s], kb * BK, n0, b, p, T.b_mat);
      }
    }
  } else if (warp == 1 && lane == 0 && n_iters > 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t id_pos = idesc_f16(BM, BNT, 0), id_neg = idesc_f16(BM, BNT, 1);
    const uint32_t acc_re = tmem, acc_im = tmem + 256;
    bool first = true;
    for (int it = 0; it < n_iters; ++it) {
      const int s = it % nstage;
      const uint32_t ph = (uint32_t)((it / nstage) & 1);
      if (!mbar_wait(&full[s], ph, e.err, abort_flag)) break;
      tc_fence_after();
      const Term T = d.t[it / nkb];
      const uint32_t sa = smem_u32(smem + s * stage_bytes);
      const uint32_t sb = sa + npl * A_TILE_BYTES;
#pragma unroll
      for (int k16 = 0; k16 < BK / 16; ++k16) {
        const uint32_t ko = k16 * 32;   // bytes along the 64-byte row
        auto A = [&](int p) { return sw64_desc(sa + p * A_TILE_BYTES + ko); };
        auto B = [&](int p) { return sw64_desc(sb + p * BTB + ko); };
        const uint32_t acc = first ? 0u : 1u;
        if (!d.complex_mode) {
          const uint32_t id = T.sign < 0 ? id_neg : id_pos;
          umma_f16(acc_re, A(0), B(0), id, acc);
          umma_f16(acc_re, A(0), B(1), id, 1u);
          umma_f16(acc_re, A(1), B(0), id, 1u);
        } else if (SPLIT) {
          // accumulators (64 columns each): rr hi*hi, rr hi*lo+lo*hi, ii .., .., ri .., ..,
          // ir .., ..: every truncating chain is a third to a sixth as long
          const int sa_ = T.a_conj ? -1 : 1, sb_ = T.b_conj ? -1 : 1;
          const int s_rr = T.sign, s_ii = -T.sign * sa_ * sb_;
          const int s_ri = T.sign * sb_, s_ir = T.sign * sa_;
          const uint32_t irr = s_rr < 0 ? id_neg : id_pos, iii = s_ii < 0 ? id_neg : id_pos;
          const uint32_t iri = s_ri < 0 ? id_neg : id_pos, iir = s_ir < 0 ? id_neg : id_pos;
          umma_f16(tmem + 0 * BNT, A(0), B(0), irr, acc);
          umma_f16(tmem + 1 * BNT, A(0), B(1), irr, acc);
          umma_f16(tmem + 1 * BNT, A(1), B(0), irr, 1u);
          umma_f16(tmem + 2 * BNT, A(2), B(2), iii, acc);
          umma_f16(tmem + 3 * BNT, A(2), B(3), iii, acc);
          umma_f16(tmem + 3 * BNT, A(3), B(2), iii, 1u);
          umma_f16(tmem + 4 * BNT, A(0), B(2), iri, acc);
          umma_f16(tmem + 5 * BNT, A(0), B(3), iri, acc);
          umma_f16(tmem + 5 * BNT, A(1), B(2), iri, 1u);
          umma_f16(tmem + 6 * BNT, A(2), B(0), iir, acc);
          umma_f16(tmem + 7 * BNT, A(2), B(1), iir, acc);
          umma_f16(tmem + 7 * BNT, A(3), B(0), iir, 1u);
        } else {
          // planes 0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo
          const int sa_ = T.a_conj ? -1 : 1, sb_ = T.b_conj ? -1 : 1;
          const int s_rr = T.sign, s_ii = -T.sign * sa_ * sb_;
          const int s_ri = T.sign * sb_, s_ir = T.sign * sa_;
          const uint32_t irr = s_rr < 0 ? id_neg : id_pos, iii = s_ii < 0 ? id_neg : id_pos;
          const uint32_t iri = s_ri < 0 ? id_neg : id_pos, iir = s_ir < 0 ? id_neg : id_pos;
          umma_f16(acc_re, A(0), B(0), irr, acc);
          umma_f16(acc_re, A(0), B(1), irr, 1u);
          umma_f16(acc_re, A(1), B(0), irr, 1u);
          umma_f16(acc_re, A(2), B(2), iii, 1u);
          umma_f16(acc_re, A(2), B(3), iii, 1u);
          umma_f16(acc_re, A(3), B(2), iii, 1u);
          umma_f16(acc_im, A(0), B(2), iri, acc);
          umma_f16(acc_im, A(0), B(3), iri, 1u);
          umma_f16(acc_im, A(1), B(2), iri, 1u);
          umma_f16(acc_im, A(2), B(0), iir, 1u);
          umma_f16(acc_im, A(2), B(1), iir, 1u);
          umma_f16(acc_im, A(3), B(0), iir, 1u);
        }
        first = false;
      }
      umma_commit(&empty[s]);
    }
    umma_commit(accb);
  } else if (warp >= 2) {
    // ---------------- epilogue ----------------
    const int q = warp & 3;                 // TMEM lane quarter of this warp
    const int m = m0 + 32 * q + lane;
    bool ok = true;
    if (n_iters > 0) ok = mbar_wait(accb, 0, e.err, abort_flag);
    tc_fence_after();
    if (ok) {
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
      for (int c = 0; c < BNT / 16; ++c) {
        float re[16], im[16];
        if (SPLIT && n_iters > 0) {
          float t0[16], t1[16];
          tmem_ld16(lane_addr + 0 * BNT + c * 16, re);
          tmem_ld16(lane_addr + 1 * BNT + c * 16, t0);
#pragma unroll
          for (int j = 0; j < 16; ++j) re[j] += t0[j];
          tmem_ld16(lane_addr + 2 * BNT + c * 16, t0);
          tmem_ld16(lane_addr + 3 * BNT + c * 16, t1);
#pragma unroll
          for (int j = 0; j < 16; ++j) re[j] += t0[j] + t1[j];
          tmem_ld16(lane_addr + 4 * BNT + c * 16, im);
          tmem_ld16(lane_addr + 5 * BNT + c * 16, t0);
#pragma unroll
          for (int j = 0; j < 16; ++j) im[j] += t0[j];
          tmem_ld16(lane_addr + 6 * BNT + c * 16, t0);
          tmem_ld16(lane_addr + 7 * BNT + c * 16, t1);
#pragma unroll
          for (int j = 0; j < 16; ++j) im[j] += t0[j] + t1[j];
        } else if (n_iters > 0) {
          tmem_ld16(lane_addr + c * 16, re);
          if (d.complex_mode) tmem_ld16(lane_addr + 256 + c * 16, im);
          else {
#pragma unroll
            for (int j = 0; j < 16; ++j) im[j] = 0.f;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) re[j] = im[j] = 0.f;
        }
        epilogue_chunk(d, e, b, m, n0 + c * 16, re, im);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, ncols);
  }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

static int make_map(const TcPlanes& t, int box_rows, CUtensorMap* m) {
  auto fn = encode_fn();
  if (!fn) return fail(SBE_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
  if (t.K % 8 != 0) return fail(SBE_ERR_UNSUPPORTED, "plane K must be a multiple of 8");
  cuuint64_t dims[5] = {(cuuint64_t)t.K, (cuuint64_t)t.rows, (cuuint64_t)t.batch,
                        (cuuint64_t)t.nplanes, (cuuint64_t)t.nmat};
  cuuint64_t row = (cuuint64_t)t.K * 2;
  cuuint64_t strides[4] = {row, row * t.rows, row * t.rows * t.batch,
                           row * t.rows * t.batch * t.nplanes};
  cuuint32_t box[5] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows, 1, 1, 1};
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, (void*)t.ptr, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(SBE_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return SBE_OK;
}

int tc_make_maps(const TcPlanes& a, const TcPlanes& b, CUtensorMap* ma, CUtensorMap* mb) {
  int rc = make_map(a, tc::BM, ma);
  if (rc) return rc;
  return make_map(b, tc::BN, mb);
}

static const int kTcSmem = 192 * 1024 + 1024 + 256;

int tc_gemm_init() {
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(tc::k_tc_gemm<tc::BN, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess ||
        cudaFuncSetAttribute(tc::k_tc_gemm<tc::BN_SPLIT, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess)
      return fail(SBE_ERR_CUDA, "tc_gemm: cannot raise the shared-memory limit");
    attr = true;
  }
  return SBE_OK;
}

int tc_gemm_launch(const tc::GemmDesc& d, const CUtensorMap& ma, const CUtensorMap& mb,
                   const tc::EpiArgs& e, cudaStream_t s) {
  const int smem = kTcSmem;
  int rc = tc_gemm_init();
  if (rc) return rc;
  if (d.split) {
    if (!d.complex_mode || d.kskip)
      return fail(SBE_ERR_ARG, "tc_gemm: split-accumulator mode is complex and unskipped only");
    dim3 grid((d.N + tc::BN_SPLIT - 1) / tc::BN_SPLIT, (d.M + tc::BM - 1) / tc::BM, d.batch);
    tc::k_tc_gemm<tc::BN_SPLIT, true><<<grid, tc::NUM_THREADS, smem, s>>>(ma, mb, d, e);
  } else {
    dim3 grid((d.N + tc::BN - 1) / tc::BN, (d.M + tc::BM - 1) / tc::BM, d.batch);
    tc::k_tc_gemm<tc::BN, false><<<grid, tc::NUM_THREADS, smem, s>>>(ma, mb, d, e);
  }
  return cuda_check(cudaGetLastError(), "tc_gemm launch");
}

int tc_make_map_split(const TcPlanes& b, CUtensorMap* mb) { return make_map(b, tc::BN_SPLIT, mb); }

}  // namespace sbe
