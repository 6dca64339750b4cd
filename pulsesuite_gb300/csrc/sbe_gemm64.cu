// Plain FP64 SIMT complex GEMMs of the SBE right-hand side (the drop-in path and
// the on-device FP64 reference of the mixed-precision path).
//
// dpdt/dCdt/dDdt (SBEs.py:1942-1965, 2309-2327, 2607-2625) are sums of four
// complex matrix products each (p stored [kh][ke]):
//   dP = (Hhh p + p Hee^T - Heh^T C - D^T Heh^T + Heh^T)/(i hbar) - (gE+gH) p
//        + (A p + p B^T)                      [off-diagonal dephasing, A,B real]
//   dC = (C Hee^T - Hee^T C + p^H Heh^T - conj(Heh) p)/(i hbar)
//   dD = (D Hhh^T - Hhh^T D + conj(p) Heh - Heh^H p^T)/(i hbar)
// One kernel evaluates out = sum_t alpha_t op(A_t) op(B_t) (+ epilogue) with
// 64x64 output tiles, 8-deep K slabs in shared memory and 4x4 outputs per thread.
#include "sbe_ctx.cuh"

namespace sbe {

constexpr int BM = 64, BN = 64, BK = 8;

struct GemmShape {   // per-launch shape rule
  int mode;          // 0: square Nk x Nk x Nk;  1: sources Nk x Nr x Nk (B = Expikr)
};

__device__ inline double2 load_op(const void* X, int op, int real, int nrow_ld, int r, int c) {
  // element (r, c) of op(X); X is row-major with leading dimension nrow_ld
  long long idx = (op == OP_N || op == OP_C) ? (long long)r * nrow_ld + c : (long long)c * nrow_ld + r;
  double2 v;
  if (real) v = make_double2(static_cast<const double*>(X)[idx], 0.0);
  else v = static_cast<const double2*>(X)[idx];
  if (op == OP_C || op == OP_H) v.y = -v.y;
  return v;
}

struct GemmArgs {
  GemmBatch b;
  int mode;
  int nk_single;
  int batched;
  const double2* expikr;
};

__global__ void __launch_bounds__(256) k_gemm64(const WireDev* wires, GemmArgs g) {
  int nk, nr;
  long long off_mat = 0, off_kr = 0, off_vec = 0;
  if (g.batched) {
    const WireDev& W = wires[g.b.w_only >= 0 ? g.b.w_only : blockIdx.z];
    if (g.b.flag_mask && (W.flags & g.b.flag_mask) != g.b.flag_mask) return;
    nk = W.nk;
    nr = W.nr;
    off_mat = W.off_mat;
    off_kr = W.off_kr;
    off_vec = W.off_vec;
  } else {
    nk = g.nk_single;
    nr = 2 * nk + 2;
  }
  const int M = nk, K = nk, N = (g.mode == 1) ? nr : nk;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  if (m0 >= M || n0 >= N) return;
  __shared__ double2 As[BK][BM + 1];
  __shared__ double2 Bs[BK][BN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);

  for (int t = 0; t < g.b.nterms; ++t) {
    const Term T = g.b.t[t];
    const char* Abase = static_cast<const char*>(T.A) + off_mat * (T.realA ? 8 : 16);
    const void* Ap = Abase;
    const void* Bp;
    int ldb;
    if (g.mode == 1) {
      Bp = g.expikr + off_kr;
      ldb = nr;
    } else {
      Bp = static_cast<const char*>(T.B) + off_mat * 16;
      ldb = nk;
    }
    for (int k0 = 0; k0 < K; k0 += BK) {
      // A tile: BM x BK, 512 elements, 2 per thread
      for (int e = threadIdx.x; e < BM * BK; e += 256) {
        int mm = e / BK, kk = e % BK;
        int gm = m0 + mm, gk = k0 + kk;
        double2 v = make_double2(0.0, 0.0);
        if (gm < M && gk < K) v = cmul(T.alpha, load_op(Ap, T.opA, T.realA, nk, gm, gk));
        As[kk][mm] = v;
      }
      for (int e = threadIdx.x; e < BK * BN; e += 256) {
        int kk = e / BN, nn = e % BN;
        int gk = k0 + kk, gn = n0 + nn;
        double2 v = make_double2(0.0, 0.0);
        if (gk < K && gn < N) v = load_op(Bp, T.opB, 0, ldb, gk, gn);
        Bs[kk][nn] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        double2 a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            acc[i][j].x = fma(a[i].x, b[j].x, fma(-a[i].y, b[j].y, acc[i][j].x));
            acc[i][j].y = fma(a[i].x, b[j].y, fma(a[i].y, b[j].x, acc[i][j].y));
          }
      }
      __syncthreads();
    }
  }
  const double ih = 1.0 / kHbar;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int m = m0 + ty + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int n = n0 + tx + 16 * j;
      if (n >= N) continue;
      double2 v = acc[i][j];
      if (g.b.epi == 1) {
        // + Heh[ke][kh]/(i hbar) - (gE[ke] + gH[kh]) p[kh][ke]   (m = kh, n = ke)
        double2 h = g.b.Heh[off_mat + (long long)n * nk + m];
        double2 p = g.b.P[off_mat + (long long)m * nk + n];
        double gam = g.b.gamE[off_vec + n] + g.b.gamH[off_vec + m];
        v.x += h.y * ih - gam * p.x;
        v.y += -h.x * ih - gam * p.y;
        if (g.b.offp) {
          double2 o = g.b.offp[off_mat + (long long)m * nk + n];
          v.x += o.y * ih;
          v.y += -o.x * ih;
        }
      }
      g.b.out[(g.mode == 1 ? off_kr : off_mat) + (long long)m * N + n] = v;
    }
  }
}

void launch_gemm64(const WireDev* d_wires, int nw, int nk_max, const GemmBatch& b, bool batched,
                   int nk_single, cudaStream_t s) {
  GemmArgs g;
  g.b = b;
  g.mode = 0;
  g.nk_single = nk_single;
  g.batched = batched ? 1 : 0;
  g.expikr = nullptr;
  int nk = batched ? nk_max : nk_single;
  dim3 grid((nk + BN - 1) / BN, (nk + BM - 1) / BM, (batched && b.w_only < 0) ? nw : 1);
  k_gemm64<<<grid, 256, 0, s>>>(d_wires, g);
}

void launch_sources_gemm64(SbeCtx* c, const GemmBatch& b, cudaStream_t s) {
  GemmArgs g;
  g.b = b;
  g.mode = 1;
  g.nk_single = 0;
  g.batched = 1;
  g.expikr = c->expikr;
  dim3 grid((c->nr_max + BN - 1) / BN, (c->nk_max + BM - 1) / BM, b.w_only >= 0 ? 1 : c->nw);
  k_gemm64<<<grid, 256, 0, s>>>(c->d_wires, g);
}

static inline Term term(const void* A, int opA, const void* B, int opB, double2 alpha,
                        int realA = 0) {
  Term t;
  t.A = A;
  t.B = B;
  t.opA = opA;
  t.opB = opB;
  t.realA = realA;
  t.alpha = alpha;
  return t;
}

// Full RHS of every wire of the context from the Hamiltonians in c->Heh/Hee/Hhh,
// the rates in c->gamE/gamH and the dephasing matrices c->dA/dB.
void launch_rhs64_ctx(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                      double2* dP, double2* dC, double2* dD, cudaStream_t s) {
  const double ih = 1.0 / kHbar;
  const double2 pos = make_double2(0.0, -ih);  //  1/(i hbar)
  const double2 neg = make_double2(0.0, ih);   // -1/(i hbar)
  const double2 one = make_double2(1.0, 0.0);
  GemmBatch b{};
  b.nterms = 0;
  b.t[b.nterms++] = term(c->Hhh, OP_N, P, OP_N, pos);
  b.t[b.nterms++] = term(D, OP_T, c->Heh, OP_T, neg);
  b.t[b.nterms++] = term(P, OP_N, c->Hee, OP_T, pos);
  b.t[b.nterms++] = term(c->Heh, OP_T, C, OP_N, neg);
  if (c->any_offdiag) {
    b.t[b.nterms++] = term(c->dA, OP_N, P, OP_N, one);
    b.t[b.nterms++] = term(P, OP_N, c->dB, OP_T, one);
  }
  b.out = dP;
  b.epi = 1;
  b.Heh = c->Heh;
  b.P = P;
  b.gamE = c->gamE;
  b.gamH = c->gamH;
  b.offp = nullptr;
  launch_gemm64(c->d_wires, c->nw, c->nk_max, b, true, 0, s);

  GemmBatch bc{};
  bc.t[bc.nterms++] = term(C, OP_N, c->Hee, OP_T, pos);
  bc.t[bc.nterms++] = term(c->Hee, OP_T, C, OP_N, neg);
  bc.t[bc.nterms++] = term(P, OP_H, c->Heh, OP_T, pos);
  bc.t[bc.nterms++] = term(c->Heh, OP_C, P, OP_N, neg);
  bc.out = dC;
  bc.epi = 0;
  launch_gemm64(c->d_wires, c->nw, c->nk_max, bc, true, 0, s);

  GemmBatch bd{};
  bd.t[bd.nterms++] = term(D, OP_N, c->Hhh, OP_T, pos);
  bd.t[bd.nterms++] = term(c->Hhh, OP_T, D, OP_N, neg);
  bd.t[bd.nterms++] = term(P, OP_C, c->Heh, OP_N, pos);
  bd.t[bd.nterms++] = term(c->Heh, OP_H, P, OP_T, neg);
  bd.out = dD;
  bd.epi = 0;
  launch_gemm64(c->d_wires, c->nw, c->nk_max, bd, true, 0, s);
}

}  // namespace sbe
