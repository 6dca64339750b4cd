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
// Tiles: BM = 128 rows, BN = 256 or 128 columns, BK = 32 (64-byte rows,
// K-major on both operands, 64-byte swizzle).  The planes live in global memory
// in the tile layout of PlaneSet: every operand tile is one contiguous chunk,
// moved to shared memory with a single cp.async.bulk.
//
// The kernel is persistent: one CTA per SM walks a list of output tiles that
// may span several GEMMs of the same shape class (jobs) and K parts of each.
// Warp roles: warp 0 issues the bulk copies through a ring of stages that runs
// on across tiles, warp 1 owns tensor memory and issues tcgen05.mma from one
// thread, warps 2-9 read the accumulators (tcgen05.ld; two warps per TMEM lane
// quarter, one per column half) and run the epilogue of tile i while the copies
// (and, when the accumulators fit twice in tensor memory, the MMAs) of tile
// i + 1 proceed.
#pragma once
#include <cuda_fp16.h>
#include <cstdint>

namespace sbe {
namespace tc {

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int BN_HH = 128;     // N tile of the hi*hi mode (MMA N = 256 over re and im of B)
constexpr int BK = 32;
constexpr int A_TILE_BYTES = BM * BK * 2;   // 8 KB
constexpr int B_TILE_BYTES = BN * BK * 2;   // 16 KB
constexpr int NUM_THREADS = 320;   // producer warp, MMA warp, 8 epilogue warps
constexpr int MAX_TERMS = 4;
constexpr int MAX_JOBS = 32;   // jobs per launch (e.g. three GEMMs for each of ten Nk buckets)
// bounded waits: an iteration limit after which the kernel flags an error
constexpr long long WAIT_LIMIT = 1ll << 28;

// Operand planes in the tile layout.  Slab (mat, plane, batch) holds a rows x K
// FP16 matrix as K-blocks of 32 columns; K-block kb stores all rows_pad rows of
// 64 bytes contiguously, swizzled in 512-byte atoms (16-byte chunk c of row r at
// chunk c ^ ((r >> 1) & 3)), which is the shared-memory image the tensor core's
// 64-byte-swizzle K-major descriptor reads.  A tile of R rows starting at a row
// multiple of 64 in K-block kb is then the contiguous R x 64 bytes at
// (kb * rows_pad + row0) * 32 elements.  rows_pad is a multiple of 256, K_pad of
// 32; the padding is zero.
struct PlaneSet {
  __half* ptr;
  int nmat, nplanes, batch, rows, K, rows_pad, K_pad;
};

__host__ __device__ inline long long plane_slab(const PlaneSet& p) {
  return (long long)p.rows_pad * p.K_pad;
}
// element offset of (r, k) within a slab
__host__ __device__ inline long long tile_off(int rows_pad, int r, int k) {
  const long long byte = ((long long)(k >> 5) * rows_pad + r) * 64 + (k & 31) * 2;
  return (byte ^ (((byte >> 7) & 3) << 4)) >> 1;
}
// element offset of (r, k) of slab (mat, plane, batch)
__host__ __device__ inline long long plane_elem(const PlaneSet& p, int mat, int plane, int b,
                                                int r, int k) {
  return ((long long)(mat * p.nplanes + plane) * p.batch + b) * plane_slab(p) +
         tile_off(p.rows_pad, r, k);
}
// element offset of the 16-byte chunk j (columns 8j .. 8j + 7 of K-block kb) of
// row r in slab (mat, plane, batch): the chunk stays contiguous under the swizzle
__host__ __device__ inline long long chunk_elem(const PlaneSet& p, int mat, int plane, int b,
                                                int r, int kb, int j) {
  return ((long long)(mat * p.nplanes + plane) * p.batch + b) * plane_slab(p) +
         ((long long)kb * p.rows_pad + r) * 32 + 8 * (j ^ ((r >> 1) & 3));
}
inline PlaneSet make_planeset(__half* ptr, int nmat, int nplanes, int batch, int rows, int K) {
  PlaneSet p{ptr, nmat, nplanes, batch, rows, K, (rows + 255) / 256 * 256, (K + 31) / 32 * 32};
  return p;
}
inline size_t planeset_bytes(const PlaneSet& p) {
  return sizeof(__half) * (size_t)p.nmat * p.nplanes * p.batch * plane_slab(p);
}

// One term of a GEMM: accumulate sign * op(A[a_mat]) * op(B[b_mat]).
struct Term {
  int a_mat, b_mat;   // matrix index in the A / B plane tensors
  int a_conj, b_conj; // complex conjugate (complex mode)
  int sign;           // +1 or -1
};

enum Epi : int {
  EPI_RAW = 0,      // out[b][m][n] = (re, im) * 2^-escale[b] as FP64 (self-test)
  EPI_F32 = 1,      // outf[b][m][n] = acc * 2^-escale[b] as FP32 (real mode)
  EPI_RAWF = 2,     // outf2[b][m][n] = (re, im) * 2^-escale[b] as FP32 complex
};

struct EpiArgs {
  int kind;
  double2* out;               // EPI_RAW output (per batch stride out_bstride)
  float* outf;                // EPI_F32 output (per batch stride out_bstride)
  float2* outf2;              // EPI_RAWF output (per batch stride out_bstride)
  long long out_bstride;
  long long ks_stride;        // output offset (elements) between the K parts of a split-K GEMM
  int ldo;                    // output row stride in elements (0: N)
  const int* escale;          // per batch exponent of the product scale (e_A + e_B)
  int* err;                   // error flag (bounded waits)
  // EPI_F32 of the exchange products (0: off): column n of row m is component
  // n & 1 of diagonal dd = n >> 1, stored un-sheared as component n & 1 of the
  // complex element [m][m + dd - (unshear - 1)] of an unshear x unshear matrix
  // (row stride ldo floats); elements outside that matrix are not stored
  int unshear;
};

enum Mode : int { MODE_FULL = 0, MODE_HH = 1 };

struct GemmDesc {
  int M, N, K;                // per batch
  int complex_mode;           // 1: 4 planes per matrix, 2 accumulators; 0: 2 planes, 1 acc
  int nterms;
  Term t[MAX_TERMS];
  int batch;
  int kskip;                  // exchange: K range limited by the sheared N tile
  int nk_shear;               // exchange: Nk of the shear
  // Product modes.  MODE_FULL: hi*hi + hi*lo + lo*hi (N tile 256); with xonly set
  // (complex only) the hi*hi products are left out.  MODE_HH (complex only, B never
  // conjugated): the hi*hi products alone, N tile 128, one FP32 accumulator per real
  // product (rr, ri, ir, ii: one MMA of N = 256 per A plane over B's re and im
  // tiles), combined in the epilogue; 512 TMEM columns, one tile in flight.  The
  // tensor core's accumulation truncates at every MMA, so a product whose result is a
  // small difference of large sums (the W - W^H form of dC, dD) takes its hi*hi part
  // in MODE_HH with split-K (short truncating chains, kseq) and its hi*lo + lo*hi
  // part, 2^-11 smaller, through xonly.
  int mode;
  int xonly;
  // split-K: the K blocks are cut into ksplit parts, each a separate output tile
  // written at out + ks * ks_stride (ksplit 0 counts as 1)
  int ksplit;
  // with ksplit > 1 (EPI_RAWF only): the parts of an output tile run in sequence in
  // one CTA, each its own accumulation chain, and the epilogue sums them in part
  // order into one output, ((p0 + p1) + p2) + ..., in FP32 (the first part stores,
  // each later part reads back what the same thread stored and adds to it)
  int kseq;
  // EPI_RAWF: add every part (the first one too) to what the output already holds,
  // e.g. the cross terms another launch wrote there before
  int kacc;
  // N tile of MODE_FULL: 256 (0 = the default) or 128; with 128 a complex tile's
  // accumulators take 256 TMEM columns, so two tiles are in flight (the epilogue of
  // one overlaps the MMAs of the next) at twice the operand loads per output
  int bn;
  PlaneSet A, B;              // operand planes (A: M rows, B: N rows, both K-major)
};

struct GemmJob {
  GemmDesc d;
  EpiArgs e;
};

// one launch: the concatenated tile lists of njobs jobs (same mode and complex flag),
// passed as one __grid_constant__ kernel parameter
struct GemmLaunch {
  GemmJob job[MAX_JOBS];
  long long tile_base[MAX_JOBS + 1];
  int njobs;
  int* sched;                 // tile counter of this launch (zeroed before it)
};
static_assert(sizeof(GemmLaunch) <= 32000, "kernel parameter space (32 KB) exceeded");

}  // namespace tc

// Host API of the engine.
int tc_gemm_launch(const tc::GemmJob* jobs, int njobs, cudaStream_t s);
int tc_gemm_launch(const tc::GemmDesc& d, const tc::EpiArgs& e, cudaStream_t s);
// One launch whose bounded wait gives up (~2 s): raises *err, *gave_up = 1.
int tc_wait_selftest(int* err, int* gave_up, cudaStream_t s);
int tc_gemm_init();

}  // namespace sbe
