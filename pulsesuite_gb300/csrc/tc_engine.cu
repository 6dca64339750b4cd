// tcgen05 / bulk-copy / TMEM split-precision GEMM engine (see tc_gemm.cuh).
#include "sbe_ctx.cuh"
#include "fp_bits.cuh"
#include "tc_gemm.cuh"
#include "tc_ptx.cuh"

namespace sbe {
namespace tc {

// ---------------------------------------------------------------------------
// epilogues

// Epilogue parameters of one tile, read from the launch parameters once per tile
// (values in registers: a parameter read inside the chunk loop would put a
// dependent load into every chunk).  Output pointers are offset to the tile's
// batch entry and K part.
struct EpiTile {
  int kind, M, N, ld, cplx, es, unshear;
  float* of;      // EPI_F32
  float2* of2;    // EPI_RAWF
  double2* od;    // EPI_RAW
};

__device__ __forceinline__ EpiTile epi_tile(const GemmDesc& d, const EpiArgs& e, int b, int ks) {
  EpiTile t;
  t.kind = e.kind;
  t.M = d.M;
  t.N = d.N;
  t.ld = e.ldo > 0 ? e.ldo : d.N;
  t.cplx = d.complex_mode;
  t.es = -e.escale[b];
  t.unshear = e.unshear;
  const long long off = (long long)ks * e.ks_stride + (long long)b * e.out_bstride;
  t.of = e.outf ? e.outf + off : nullptr;
  t.of2 = e.outf2 ? e.outf2 + off : nullptr;
  t.od = e.out ? e.out + off : nullptr;
  return t;
}

// Epilogue of one 16-column chunk (columns n0 .. n0 + 15) of the warp's 32 rows
// mrow0 + lane.  re[j], im[j] arrive in the TMEM orientation (lane = row, j =
// column); the chunk is transposed through the warp's shared-memory scratch
// (32 x 16 float2, column slot j ^ (row & 15) so that both passes are free of
// bank conflicts) so that every global store runs along n: in the column pass
// lanes 0-15 and 16-31 take the columns of two rows at a time.  The column pass
// reads its 16 values into registers before it stores (shared and global
// accesses through generic pointers would otherwise serialise on the
// shared-memory latency).
__device__ __forceinline__ void epilogue_chunk(const EpiTile& t, int mrow0, int n0, float* re,
                                               float* im, float2* scr, bool accumulate) {
  const int lane = threadIdx.x & 31;
  const int es = t.es;
  // ---- row pass
  if (t.kind != EPI_RAW) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      re[j] = f32_ldexp(re[j], es);
      im[j] = f32_ldexp(im[j], es);
    }
  }
#pragma unroll
  for (int j = 0; j < 16; ++j) scr[lane * 16 + (j ^ (lane & 15))] = make_float2(re[j], im[j]);
  __syncwarp();
  // ---- column pass: lane -> column j, rows rh, rh + 2, ...
  const int j = lane & 15, rh = lane >> 4;
  float2 v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int r = 2 * i + rh;
    v[i] = scr[r * 16 + (j ^ (r & 15))];
  }
  __syncwarp();
  const int n = n0 + j;
  const int rmax = min(32, t.M - mrow0);
  if (n >= t.N) return;
  const long long base = (long long)(mrow0 + rh) * t.ld + n;
  const long long rs = 2 * (long long)t.ld;
  if (t.kind == EPI_RAWF) {
    float2* o = t.of2 + base;
    if (accumulate) {
      // a later K part of a kseq tile: add to the running sum this thread stored
      float2 pv[16];
#pragma unroll
      for (int i = 0; i < 16; ++i)
        if (2 * i + rh < rmax) pv[i] = o[i * rs];
#pragma unroll
      for (int i = 0; i < 16; ++i)
        if (2 * i + rh < rmax) o[i * rs] = make_float2(pv[i].x + v[i].x, pv[i].y + v[i].y);
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i)
        if (2 * i + rh < rmax) o[i * rs] = v[i];
    }
  } else if (t.kind == EPI_F32 && t.unshear) {
    // row r = mrow0 + rh + 2i, diagonal n >> 1: complex column k2 = r + (n >> 1) -
    // (unshear - 1); consecutive lanes store consecutive floats of one row
    const int k20 = mrow0 + rh + (n >> 1) - (t.unshear - 1);
    float* o = t.of + (long long)(mrow0 + rh) * t.ld + 2 * k20 + (n & 1);
    const long long rs2 = 2 * (long long)t.ld + 4;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int k2 = k20 + 2 * i;
      if (2 * i + rh < rmax && k2 >= 0 && k2 < t.unshear) o[i * rs2] = v[i].x;
    }
  } else if (t.kind == EPI_F32) {
    float* o = t.of + base;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (2 * i + rh < rmax) o[i * rs] = v[i].x;
  } else {
    // EPI_RAW: exact widening and power-of-two scaling on the integer pipe
    double2* o = t.od + base;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (2 * i + rh < rmax)
        o[i * rs] = make_double2(f32_to_f64_scaled(v[i].x, es),
                                 t.cplx ? f32_to_f64_scaled(v[i].y, es) : 0.0);
  }
}

// ---------------------------------------------------------------------------
// the kernel

// One output tile of the launch's tile list.
struct TileInfo {
  int job, b, m0, n0, ks, kb_begin, nkb, n_iters;
  int nparts;  // K parts run in sequence in this tile (kseq), else 1
  bool dead;   // exchange tile whose outputs all lie outside the un-sheared matrix
};

// K blocks [begin, end) of part p of nparts over all K blocks
__device__ __forceinline__ void part_range(int nkb_all, int p, int nparts, int* b, int* e) {
  *b = p * nkb_all / nparts;
  *e = (p + 1) * nkb_all / nparts;
}

template <int BNT>
__device__ __forceinline__ TileInfo tile_info(const GemmLaunch& L, long long t) {
  TileInfo ti;
  // job of tile t: the last j with tile_base[j] <= t (binary search)
  int j = 0, hi = L.njobs - 1;
  while (j < hi) {
    const int mid = (j + hi + 1) >> 1;
    if (L.tile_base[mid] <= t)
      j = mid;
    else
      hi = mid - 1;
  }
  const GemmDesc& d = L.job[j].d;
  long long r = t - L.tile_base[j];
  const int tn = (d.N + BNT - 1) / BNT, tm = (d.M + BM - 1) / BM;
  ti.job = j;
  ti.n0 = (int)(r % tn) * BNT;
  r /= tn;
  ti.m0 = (int)(r % tm) * BM;
  r /= tm;
  ti.b = (int)(r % d.batch);
  ti.ks = (int)(r / d.batch);
  // K blocks of this part (kseq: of the whole K range; the parts are cut in the loops)
  const int nkb_all = (d.K + BK - 1) / BK;
  const int ksplit = (d.ksplit > 1 && !d.kseq) ? d.ksplit : 1;
  ti.nparts = (d.ksplit > 1 && d.kseq) ? d.ksplit : 1;
  int kb_begin = ti.ks * nkb_all / ksplit, kb_end = (ti.ks + 1) * nkb_all / ksplit;
  if (d.kskip) {
    // the sheared exchange operand is zero outside the band of this N tile
    const int nk = d.nk_shear;
    const int dd_lo = ti.n0 / 2, dd_hi = min((ti.n0 + BNT) / 2, 2 * nk - 1) - 1;
    const int dlo = dd_lo - (nk - 1), dhi = dd_hi - (nk - 1);
    const int tlo = max(0, -dhi), thi = min(nk - 1, nk - 1 - dlo);
    kb_begin = max(kb_begin, tlo / BK);
    kb_end = (thi >= tlo) ? min(kb_end, thi / BK + 1) : kb_begin;
    // output (m, dd) is element [m][m + dd - (Nk - 1)] of the Hamiltonian: the tile
    // is used only if some m + dd of it lies in [Nk - 1, 2 Nk - 2]
    const int m_hi = min(ti.m0 + BM, d.M) - 1;
    ti.dead = (dd_lo + ti.m0 > 2 * nk - 2) || (dd_hi + m_hi < nk - 1);
  } else {
    ti.dead = false;
  }
  ti.kb_begin = kb_begin;
  ti.nkb = max(0, kb_end - kb_begin);
  ti.n_iters = d.nterms * ti.nkb;
  return ti;
}

constexpr int EPI_WARPS = 8;
constexpr int SCR_BYTES = EPI_WARPS * 32 * 16 * 8;   // epilogue transpose scratch per warp
constexpr int STAGE_AREA = 192 * 1024;

template <int BNT, int MODE>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_tc_gemm(const __grid_constant__ GemmLaunch L) {
  constexpr int BTB = BNT * BK * 2;   // B tile bytes per plane
  constexpr bool HH = (MODE == MODE_HH);
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const bool cplx = L.job[0].d.complex_mode != 0;
  // planes per operand tile in shared memory (MODE_HH: re_hi, im_hi)
  const int npl = HH ? 2 : (cplx ? 4 : 2);
  const int stage_bytes = npl * (A_TILE_BYTES + BTB);
  const int nstage = min(8, STAGE_AREA / stage_bytes);
  // accumulator columns of one tile; two tiles in flight when they fit twice
  // (MODE_HH: B's re and im plane tiles lie back to back in shared memory, so one
  // MMA of N = 2 BNT per A plane forms two real products: 4 BNT columns)
  const int tile_cols = HH ? 4 * BNT : (cplx ? 2 * BNT : BNT);
  const int nbuf = tile_cols <= 256 ? 2 : 1;
  float2* scr_all = reinterpret_cast<float2*>(smem + STAGE_AREA);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGE_AREA + SCR_BYTES);
  uint64_t* empty = full + 8;
  uint64_t* tfull = empty + 8;
  uint64_t* tempty = tfull + 2;
  // tile queue: the producer takes tiles from the launch's counter (dynamic
  // scheduling) and hands each tile index to the MMA issuer and the epilogue
  uint64_t* qfull = tempty + 2;
  uint64_t* qempty = qfull + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(qempty + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* tq = abort_flag + 1;   // 4 queue entries
  int* err = L.job[0].e.err;

  const int warp = threadIdx.x / 32, lane = threadIdx.x & 31;
  const long long ntiles = L.tile_base[L.njobs];

  if (threadIdx.x == 0) {
    for (int s = 0; s < nstage; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], EPI_WARPS);   // one arrival per epilogue warp
    }
    for (int i = 0; i < 4; ++i) {
      mbar_init(&qfull[i], 1);
      mbar_init(&qempty[i], 1 + EPI_WARPS);   // the MMA issuer and each epilogue warp
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- bulk-copy producer ----------------
    long long g = 0;   // stage-ring position (runs on across tiles)
    bool ok = true;
    for (int k = 0; ok; ++k) {
      const int qs = k & 3;
      if (!mbar_wait(&qempty[qs], (uint32_t)(((k >> 2) & 1) ^ 1), err, abort_flag)) break;
      long long t = atomicAdd(L.sched, 1);
      while (t < ntiles && tile_info<BNT>(L, t).dead) t = atomicAdd(L.sched, 1);
      tq[qs] = t < ntiles ? (int)t : -1;
      mbar_arrive(&qfull[qs]);   // release: the entry is visible to the waiters
      if (t >= ntiles) break;
      const TileInfo ti = tile_info<BNT>(L, t);
      const GemmDesc& d = L.job[ti.job].d;
      // slab strides (elements) of the operand planes; K-block kb of a tile starts
      // at kb * rows_pad * BK within its slab
      const long long sA = plane_slab(d.A), sB = plane_slab(d.B);
      const long long kstepA = (long long)d.A.rows_pad * BK, kstepB = (long long)d.B.rows_pad * BK;
      const int pstep = HH ? 2 : 1;   // MODE_HH loads planes re_hi, im_hi
      // a last N tile narrower than BNT (MODE_FULL) loads only the B rows its
      // MMAs read, rounded up to the 64-row tile granule
      const int nrem = d.N - ti.n0;
      const int bbytes = (HH || nrem >= BNT) ? BTB : ((nrem + 63) & ~63) * BK * 2;
      const uint32_t tx_bytes = (uint32_t)(npl * (A_TILE_BYTES + bbytes));
      int s = (int)(g % nstage);
      uint32_t ph = (uint32_t)((g / nstage) & 1);
      for (int part = 0; ok && part < ti.nparts; ++part) {
      int kb0 = ti.kb_begin, nkb = ti.nkb;
      if (ti.nparts > 1) {
        int e_;
        part_range(ti.nkb, part, ti.nparts, &kb0, &e_);
        nkb = e_ - kb0;
        kb0 += ti.kb_begin;
      }
      for (int term = 0; ok && term < d.nterms && nkb > 0; ++term) {
        const Term T = d.t[term];
        const __half* ga0 = d.A.ptr + ((long long)T.a_mat * d.A.nplanes * d.A.batch + ti.b) * sA +
                            ((long long)kb0 * d.A.rows_pad + ti.m0) * BK;
        const __half* gb0 = d.B.ptr + ((long long)T.b_mat * d.B.nplanes * d.B.batch + ti.b) * sB +
                            ((long long)kb0 * d.B.rows_pad + ti.n0) * BK;
        const long long pA = (long long)pstep * d.A.batch * sA, pB = (long long)pstep * d.B.batch * sB;
        for (int kk = 0; kk < nkb; ++kk, ++g) {
          if (!mbar_wait(&empty[s], ph ^ 1u, err, abort_flag)) {
            ok = false;
            break;
          }
          uint8_t* sa = smem + s * stage_bytes;
          uint8_t* sb = sa + npl * A_TILE_BYTES;
          mbar_expect_tx(&full[s], tx_bytes);
          const __half* ga = ga0 + kk * kstepA;
          const __half* gb = gb0 + kk * kstepB;
          for (int p = 0; p < npl; ++p) {
            bulk_load(sa + p * A_TILE_BYTES, ga + p * pA, A_TILE_BYTES, &full[s]);
            bulk_load(sb + p * BTB, gb + p * pB, bbytes, &full[s]);
          }
          if (++s == nstage) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
      }
    }
    // no copy may still be landing in shared memory when the CTA exits: wait
    // (bounded) for the last stages issued
    for (long long q = max(0ll, g - nstage); q < g; ++q) {
      volatile int never = 0;
      mbar_wait(&full[q % nstage], (uint32_t)((q / nstage) & 1), err, &never);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    constexpr int MMA_N = HH ? 2 * BNT : BNT;
    const uint32_t id_pos_full = idesc_f16(BM, MMA_N, 0), id_neg_full = idesc_f16(BM, MMA_N, 1);
    long long g = 0;
    bool ok = true;
    int st = 0;   // accumulator sub-tiles issued (one per K part of a kseq tile)
    for (int lt = 0; ok; ++lt) {
      const int qs = lt & 3;
      if (!mbar_wait(&qfull[qs], (uint32_t)((lt >> 2) & 1), err, abort_flag)) break;
      const int t = tq[qs];
      mbar_arrive(&qempty[qs]);
      if (t < 0) break;
      const TileInfo ti = tile_info<BNT>(L, t);
      const GemmDesc& d = L.job[ti.job].d;
      const bool hh = !d.xonly;
      // a last N tile narrower than BNT (MODE_FULL): MMAs of N rounded up to 16
      const int nrem = d.N - ti.n0;
      const bool narrow = !HH && nrem < BNT;
      const uint32_t id_pos = narrow ? idesc_f16(BM, (nrem + 15) & ~15, 0) : id_pos_full;
      const uint32_t id_neg = narrow ? idesc_f16(BM, (nrem + 15) & ~15, 1) : id_neg_full;
      int s = (int)(g % nstage);
      uint32_t ph = (uint32_t)((g / nstage) & 1);
#pragma unroll 1
      for (int part = 0; ok && part < ti.nparts; ++part, ++st) {
      int nkb = ti.nkb;
      if (ti.nparts > 1) {
        int b_, e_;
        part_range(ti.nkb, part, ti.nparts, &b_, &e_);
        nkb = e_ - b_;
      }
      const int buf = st % nbuf, use = st / nbuf;
      if (use > 0 && !mbar_wait(&tempty[buf], (uint32_t)((use - 1) & 1), err, abort_flag)) {
        ok = false;
        break;
      }
      tc_fence_after();
      // accumulator columns of the tile: [re | im] (BNT each) at buf * 256
      const uint32_t acc_re = tmem + buf * 256, acc_im = acc_re + BNT;
      bool first = true;
      for (int term = 0; ok && term < d.nterms && nkb > 0; ++term) {
        const Term T = d.t[term];
        const int sa_ = T.a_conj ? -1 : 1, sb_ = T.b_conj ? -1 : 1;
        const int s_rr = T.sign, s_ii = -T.sign * sa_ * sb_;
        const int s_ri = T.sign * sb_, s_ir = T.sign * sa_;
        const uint32_t irr = s_rr < 0 ? id_neg : id_pos, iii = s_ii < 0 ? id_neg : id_pos;
        const uint32_t iri = s_ri < 0 ? id_neg : id_pos, iir = s_ir < 0 ? id_neg : id_pos;
        for (int kk = 0; kk < nkb; ++kk, ++g) {
          if (!mbar_wait(&full[s], ph, err, abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          // descriptors of the stage's planes: the start-address field (16-byte
          // units, bits 0-13) takes the plane and K offsets without carry
          const uint64_t da = sw64_desc(smem_u32(smem + s * stage_bytes));
          const uint64_t db = da + (uint64_t)((npl * A_TILE_BYTES) >> 4);
#pragma unroll
          for (int k16 = 0; k16 < BK / 16; ++k16) {
            const uint32_t ko = k16 * 2;   // 32 bytes along the 64-byte row
            auto A = [&](int p) { return da + (uint64_t)(p * (A_TILE_BYTES >> 4) + ko); };
            auto B = [&](int p) { return db + (uint64_t)(p * (BTB >> 4) + ko); };
            const uint32_t acc = first ? 0u : 1u;
            if (!cplx) {
              const uint32_t id = T.sign < 0 ? id_neg : id_pos;
              umma_f16(acc_re, A(0), B(0), id, acc);
              umma_f16(acc_re, A(0), B(1), id, 1u);
              umma_f16(acc_re, A(1), B(0), id, 1u);
            } else if (HH) {
              // planes 0 re_hi, 1 im_hi; B(0) spans B's re and im tiles.  Columns of
              // the tile's buffer: [rr | ri] from A re, [ir | -ii] from A im (B is
              // never conjugated here, so ri takes rr's sign and ii the negative of
              // ir's; the epilogue forms re = rr - (-ii), im = ri + ir)
              umma_f16(acc_re, A(0), B(0), irr, acc);
              umma_f16(acc_re + 2 * BNT, A(1), B(0), iir, acc);
            } else {
              // planes 0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo
              uint32_t ar = acc, ai = acc;
              if (hh) {
                umma_f16(acc_re, A(0), B(0), irr, ar);
                umma_f16(acc_re, A(2), B(2), iii, 1u);
                umma_f16(acc_im, A(0), B(2), iri, ai);
                umma_f16(acc_im, A(2), B(0), iir, 1u);
                ar = ai = 1u;
              }
              umma_f16(acc_re, A(0), B(1), irr, ar);
              umma_f16(acc_re, A(1), B(0), irr, 1u);
              umma_f16(acc_re, A(2), B(3), iii, 1u);
              umma_f16(acc_re, A(3), B(2), iii, 1u);
              umma_f16(acc_im, A(0), B(3), iri, ai);
              umma_f16(acc_im, A(1), B(2), iri, 1u);
              umma_f16(acc_im, A(2), B(1), iir, 1u);
              umma_f16(acc_im, A(3), B(0), iir, 1u);
            }
            first = false;
          }
          umma_commit(&empty[s]);
          if (++s == nstage) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
      if (!ok) break;
      // accumulators of this (sub-)tile complete (one without K blocks leaves tensor
      // memory untouched and its epilogue stores zeros)
      if (nkb > 0 && d.nterms > 0)
        umma_commit(&tfull[buf]);
      else
        mbar_arrive(&tfull[buf]);
      }
    }
  } else if (warp >= 2) {
    // ---------------- epilogue ----------------
    const int q = warp & 3;                 // TMEM lane quarter of this warp
    float2* scr = scr_all + (warp - 2) * (32 * 16);
    const int half = (warp - 2) >> 2;         // column half of the tile
    int st = 0;   // accumulator sub-tiles drained (one per K part of a kseq tile)
    bool stop = false;
    for (int lt = 0; !stop; ++lt) {
      const int qs = lt & 3;
      if (!mbar_wait(&qfull[qs], (uint32_t)((lt >> 2) & 1), err, abort_flag)) break;
      const int t = tq[qs];
      __syncwarp();
      if (lane == 0) mbar_arrive(&qempty[qs]);
      if (t < 0) break;
      const TileInfo ti = tile_info<BNT>(L, t);
      const GemmDesc& d = L.job[ti.job].d;
      const EpiArgs& e = L.job[ti.job].e;
      const int mrow0 = ti.m0 + 32 * q;
      const EpiTile et = epi_tile(d, e, ti.b, ti.ks);   // before the wait
#pragma unroll 1
      for (int part = 0; part < ti.nparts; ++part, ++st) {
      int nkb = ti.nkb;
      if (ti.nparts > 1) {
        int b_, e_;
        part_range(ti.nkb, part, ti.nparts, &b_, &e_);
        nkb = e_ - b_;
      }
      const int buf = st % nbuf, use = st / nbuf;
      if (!mbar_wait(&tfull[buf], (uint32_t)(use & 1), err, abort_flag)) {
        stop = true;
        break;
      }
      tc_fence_after();
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16) + buf * 256;
      const bool have = nkb > 0 && d.nterms > 0;
      constexpr int NCH = BNT / 32;   // 16-column chunks per column half
      for (int cc = 0; cc < NCH; ++cc) {
        const int c = half * NCH + cc;   // chunk of the tile
        if (ti.n0 + c * 16 >= d.N) {
          // chunk beyond the matrix: nothing to read or store
          if (cc == NCH - 1) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[buf]);
          }
          continue;
        }
        float re[16], im[16];
        if (have && HH) {
          // buffer columns [rr | ri | ir | -ii] (BNT each): re = rr + ii, im = ri + ir;
          // the four loads under one wait
          uint32_t a0[16], a1[16], a2[16], a3[16];
          tmem_ld16_nw(lane_addr + 0 * BNT + c * 16, a0);
          tmem_ld16_nw(lane_addr + 3 * BNT + c * 16, a3);
          tmem_ld16_nw(lane_addr + 1 * BNT + c * 16, a1);
          tmem_ld16_nw(lane_addr + 2 * BNT + c * 16, a2);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            re[j] = __uint_as_float(a0[j]) - __uint_as_float(a3[j]);
            im[j] = __uint_as_float(a1[j]) + __uint_as_float(a2[j]);
          }
        } else if (have) {
          tmem_ld16(lane_addr + c * 16, re);
          if (cplx) {
            tmem_ld16(lane_addr + BNT + c * 16, im);
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) im[j] = 0.f;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) re[j] = im[j] = 0.f;
        }
        if (cc == NCH - 1) {
          // last read of this tile's accumulators by this warp
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&tempty[buf]);
        }
        epilogue_chunk(et, mrow0, ti.n0 + c * 16, re, im, scr, part > 0 || d.kacc);
      }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// host side

static const int kTcSmem = 1024 + tc::STAGE_AREA + tc::SCR_BYTES + 512;

// per-launch tile counters of the dynamic scheduler (cycled; each launch zeroes its own)
static int* g_sched = nullptr;
static unsigned g_sched_seq = 0;
constexpr int kSchedSlots = 1024;

int tc_gemm_init() {
  static bool attr = false;
  if (!g_sched && cudaMalloc(&g_sched, sizeof(int) * kSchedSlots) != cudaSuccess) {
    g_sched = nullptr;
    return fail(SBE_ERR_OOM, "tc_gemm: scheduler counters");
  }
  if (!attr) {
    if (cudaFuncSetAttribute(tc::k_tc_gemm<tc::BN, tc::MODE_FULL>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess ||
        cudaFuncSetAttribute(tc::k_tc_gemm<128, tc::MODE_FULL>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess ||
        cudaFuncSetAttribute(tc::k_tc_gemm<tc::BN_HH, tc::MODE_HH>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess)
      return fail(SBE_ERR_CUDA, "tc_gemm: cannot raise the shared-memory limit");
    attr = true;
  }
  return SBE_OK;
}

static int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
  }
  return n;
}

// every bulk copy stays inside the plane sets: tiles of the launch grid lie in
// the padded rows, K-blocks in the padded K, terms in the allocated matrices
static bool job_ok(const tc::GemmDesc& d) {
  const int npl = d.complex_mode ? 4 : 2;
  bool ok = d.A.ptr && d.B.ptr && d.M > 0 && d.N > 0 && d.K > 0 && d.M <= d.A.rows &&
            d.N <= d.B.rows && d.K <= d.A.K && d.K <= d.B.K && d.batch > 0 &&
            d.batch <= d.A.batch && d.batch <= d.B.batch && d.A.nplanes >= npl &&
            d.B.nplanes >= npl && d.nterms >= 1 && d.nterms <= tc::MAX_TERMS &&
            d.A.rows_pad % 256 == 0 && d.B.rows_pad % 256 == 0 && d.A.K_pad % tc::BK == 0 &&
            d.B.K_pad % tc::BK == 0 && d.ksplit >= 0 && d.ksplit <= 64;
  for (int i = 0; ok && i < d.nterms; ++i)
    ok = d.t[i].a_mat >= 0 && d.t[i].a_mat < d.A.nmat && d.t[i].b_mat >= 0 &&
         d.t[i].b_mat < d.B.nmat;
  return ok;
}

int tc_gemm_launch(const tc::GemmJob* jobs, int njobs, cudaStream_t s) {
  int rc = tc_gemm_init();
  if (rc) return rc;
  if (njobs < 1 || njobs > tc::MAX_JOBS)
    return fail(SBE_ERR_ARG, "tc_gemm: 1 to " + std::to_string(tc::MAX_JOBS) + " jobs per launch");
  tc::GemmLaunch L{};
  L.njobs = njobs;
  const int mode = jobs[0].d.mode;
  const int cplx = jobs[0].d.complex_mode;
  if (mode != tc::MODE_FULL && mode != tc::MODE_HH) return fail(SBE_ERR_ARG, "tc_gemm: bad mode");
  const int bn = jobs[0].d.bn;
  if (bn != 0 && bn != 128 && bn != 256) return fail(SBE_ERR_ARG, "tc_gemm: N tile 128 or 256");
  const int bnt = mode == tc::MODE_HH ? tc::BN_HH : (bn == 128 ? 128 : tc::BN);
  long long nt = 0;
  for (int j = 0; j < njobs; ++j) {
    const tc::GemmDesc& d = jobs[j].d;
    if (!job_ok(d)) return fail(SBE_ERR_ARG, "tc_gemm: operand plane sets do not cover the launch");
    if (d.mode != mode || d.complex_mode != cplx || d.bn != bn)
      return fail(SBE_ERR_ARG, "tc_gemm: the jobs of a launch share one mode and N tile");
    if ((mode == tc::MODE_HH || d.xonly) && (!d.complex_mode || d.kskip))
      return fail(SBE_ERR_ARG, "tc_gemm: hi*hi and cross-term modes are complex and unskipped only");
    if (d.kskip && d.ksplit > 1) return fail(SBE_ERR_ARG, "tc_gemm: band skip and split-K exclude");
    if (mode == tc::MODE_HH)
      for (int i = 0; i < d.nterms; ++i)
        if (d.t[i].b_conj) return fail(SBE_ERR_ARG, "tc_gemm: hi*hi mode takes B unconjugated");
    L.job[j] = jobs[j];
    L.tile_base[j] = nt;
    if (d.kseq && (d.ksplit < 2 || jobs[j].e.kind != tc::EPI_RAWF))
      return fail(SBE_ERR_ARG, "tc_gemm: K parts in sequence need split-K and FP32 complex output");
    if (d.kacc && (jobs[j].e.kind != tc::EPI_RAWF || (d.ksplit > 1 && !d.kseq)))
      return fail(SBE_ERR_ARG, "tc_gemm: accumulating output needs FP32 complex output and one "
                               "tile per output");
    nt += (long long)((d.N + bnt - 1) / bnt) * ((d.M + tc::BM - 1) / tc::BM) * d.batch *
          (d.ksplit > 1 && !d.kseq ? d.ksplit : 1);
  }
  L.tile_base[njobs] = nt;
  if (nt == 0) return SBE_OK;
  L.sched = g_sched + (g_sched_seq++ % kSchedSlots);
  if (cudaMemsetAsync(L.sched, 0, sizeof(int), s) != cudaSuccess)
    return cuda_check(cudaGetLastError(), "tc_gemm scheduler reset");
  const int grid = (int)std::min<long long>(nt, num_sms());
  if (mode == tc::MODE_HH)
    tc::k_tc_gemm<tc::BN_HH, tc::MODE_HH><<<grid, tc::NUM_THREADS, kTcSmem, s>>>(L);
  else if (bnt == 128)
    tc::k_tc_gemm<128, tc::MODE_FULL><<<grid, tc::NUM_THREADS, kTcSmem, s>>>(L);
  else
    tc::k_tc_gemm<tc::BN, tc::MODE_FULL><<<grid, tc::NUM_THREADS, kTcSmem, s>>>(L);
  return cuda_check(cudaGetLastError(), "tc_gemm launch");
}

namespace tc {
// Self-test of the bounded wait: thread 0 waits, through mbar_wait, for phase 0 of a
// fresh barrier that nothing arrives on.  The wait gives up after its cycle limit
// (~2 s), sets *err and returns false; *gave_up records that.
__global__ void k_wait_selftest(int* err, int* gave_up) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0)
    *gave_up = mbar_wait(&bar, 0u, err, reinterpret_cast<volatile int*>(&abort_flag)) ? 0 : 1;
}
}  // namespace tc

int tc_wait_selftest(int* err, int* gave_up, cudaStream_t s) {
  tc::k_wait_selftest<<<1, 32, 0, s>>>(err, gave_up);
  return cuda_check(cudaGetLastError(), "tc_wait_selftest launch");
}

int tc_gemm_launch(const tc::GemmDesc& d, const tc::EpiArgs& e, cudaStream_t s) {
  tc::GemmJob j{d, e};
  return tc_gemm_launch(&j, 1, s);
}

}  // namespace sbe
