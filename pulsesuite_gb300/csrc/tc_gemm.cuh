// tcgen05 split-precision GEMM engine for sm_103a.
//
// Operands are FP16 "planes": every real matrix x (scaled by a power of two so
// that |x| <= 2^14) is stored as hi = fp16(x) and lo = fp16(x - hi); a complex
// matrix has four planes (re_hi, re_lo, im_hi, im_lo).  A real product is
// formed as A_hi B_hi + A_hi B_lo + A_lo B_hi (the lo*lo term is below the
// representation error), a complex product with the four real products of the
// textbook formula (conjugation and sign by the MMA's operand-negate bit), all
// accumulated in FP32 in tensor memory.
//
// Tiles: BM = 128 rows, BN = 256 columns, BK = 32 (64-byte rows, TMA
// SWIZZLE_64B, K-major on both operands).  Warp roles: warp 0 issues TMA loads,
// warp 1 owns tensor memory and issues tcgen05.mma from one thread, warps 2-5
// read the accumulators (tcgen05.ld) and run the epilogue.
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace sbe {
namespace tc {

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int BN_SPLIT = 64;   // N tile of the split-accumulator mode
constexpr int BK = 32;
constexpr int A_TILE_BYTES = BM * BK * 2;   // 8 KB
constexpr int B_TILE_BYTES = BN * BK * 2;   // 16 KB
constexpr int NUM_THREADS = 192;
constexpr int MAX_TERMS = 4;
// bounded waits: an iteration limit after which the kernel flags an error
constexpr long long WAIT_LIMIT = 1ll << 28;

// One term of a GEMM: accumulate sign * op(A[a_mat]) * op(B[b_mat]).
struct Term {
  int a_mat, b_mat;   // matrix index in the A / B plane tensors
  int a_conj, b_conj; // complex conjugate (complex mode)
  int sign;           // +1 or -1
};

enum Epi : int {
  EPI_RAW = 0,      // out[b][m][n] = (re, im) * 2^-(ea[b]+eb[b])      (self-test)
  EPI_RHS = 1,      // stage RHS of P, C or D (see sbe_tc.cu)
  EPI_EXCH = 2,     // exchange Hamiltonian assembly (see sbe_tc.cu)
  EPI_F32 = 3,      // outf[b][m][n] = acc * 2^-escale[b] as FP32 (real mode)
  EPI_RHSF = 4,     // stage RHS of P in FP32 (see sbe_tc.cu)
  EPI_RAWF = 5,     // outf2[b][m][n] = (re, im) * 2^-escale[b] as FP32 complex
};

struct EpiArgs {
  int kind;
  int which;                  // RHS: 0 dP, 1 dC, 2 dD;  EXCH: 0 eh, 1 ee, 2 hh
  double2* out;               // FP64 complex output (per batch stride out_bstride)
  float* outf;                // FP32 output (EPI_F32, per batch stride out_bstride)
  long long out_bstride;
  const int* escale;          // per batch exponent of the product scale (e_A + e_B)
  // RHS epilogue inputs (per batch strides = nk*nk or nk)
  const double2* X;           // the state matrix whose diagonal terms are added (P, C or D)
  const double2* Heh;         // FP64 Heh (dP only)
  const double2* dgE;         // diagonal of Hee (per batch, nk), peeled off the GEMM operand
  const double2* dgH;         // diagonal of Hhh
  const double* gamE;
  const double* gamH;
  // exchange epilogue
  const double2* Ek;          // per batch 3 x nr wire-k fields
  const double* Eenergy;      // per batch Ee or Eh
  const double2* tr;          // per batch traces [2][2nk]
  const double* vs;           // per batch screened V by d [3][nk]
  double2* H3;                // per batch Heh, Hee, Hhh (stride nk*nk, 3 consecutive blocks)
  int nk, nr;
  int lf, excitons, optics;
  double gap, ehint, dcv;
  const int* yw;              // per batch yw(w)
  const int* zsign;           // per batch (-1)^w
  int* err;                   // error flag (bounded waits)
  // FP32 outputs and inputs of EPI_RHSF / EPI_RAWF
  float2* outf2;
  const float2* hehf;         // Heh in FP32 [ke][kh] per batch
  const float2* dgf;          // peeled diagonals: [4][nw][nk] Hee hi, Hee lo, Hhh hi, Hhh lo
  const float* gamf;          // [2][nw][nk] GamE, GamH
  const float* cdf;           // [4][nw][nk] hi, lo of Re C_kk, then hi, lo of Re D_kk
  int nw;
};

struct GemmDesc {
  int M, N, K;                // per batch
  int complex_mode;           // 1: 4 planes per matrix, 2 accumulators; 0: 2 planes, 1 acc
  int nterms;
  Term t[MAX_TERMS];
  int batch;
  int kskip;                  // exchange: K range limited by the sheared N tile
  int nk_shear;               // exchange: Nk of the shear
  // split-accumulator mode (complex only): N tile 64 and eight FP32 accumulators,
  // one per (real product, hi*hi or hi*lo + lo*hi) pair, summed in the epilogue.
  // The tensor core's accumulation truncates; splitting the sums shortens each
  // truncating chain (for products whose result is a small difference of large
  // sums, e.g. the W - W^H form of dC, dD).
  int split;
  // K range override in BK blocks (kb_hi > kb_lo): a split-K partial product
  int kb_lo, kb_hi;
};

}  // namespace tc

// Host API of the engine (sbe_tc.cu).
struct TcPlanes {
  __half* ptr = nullptr;      // [mat][plane][batch][rows][K]
  int nmat = 0, nplanes = 0, batch = 0, rows = 0, K = 0;
};

int tc_make_maps(const TcPlanes& a, const TcPlanes& b, CUtensorMap* ma, CUtensorMap* mb);
// tensor map of a B operand for the split-accumulator mode (64-row box)
int tc_make_map_split(const TcPlanes& b, CUtensorMap* mb);
int tc_gemm_launch(const tc::GemmDesc& d, const CUtensorMap& ma, const CUtensorMap& mb,
                   const tc::EpiArgs& e, cudaStream_t s);

}  // namespace sbe
