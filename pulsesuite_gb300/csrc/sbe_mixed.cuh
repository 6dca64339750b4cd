// Mixed-precision workspace of a context (shared by sbe_tc.cu and the tile
// autotuner): the wires of one Nk form a bucket, contiguous in every packed buffer.
#pragma once
#include <vector>

#include "sbe_ctx.cuh"
#include "tc_gemm.cuh"

namespace sbe {

struct Mixed {
  int nk = 0, nw = 0, nr = 0;
  int first = 0;                          // position of its first wire in the layout order
  long long bm = 0, bv = 0, br = 0, bkr = 0;  // packed offsets of its first wire
  WireDev* dw = nullptr;                  // its wires in layout order (device)
  // N tile of the exchange, commutator and source GEMMs (indexed by JobKind; 0 =
  // the engine's default of 256; the hi*hi mode has its own fixed tile), chosen by
  // sbe_autotune
  int bn[4] = {0, 0, 0, 0};
  // K parts of the hi*hi products of W and V (split-K: shorter truncating FP32
  // chains; the parts are summed in order by the GEMM epilogue); 1 to 8, by default 2
  // below Nk = 256, 4 below Nk = 1024 and 8 from there on
  int hs = 2;
  tc::PlaneSet pl{}, tp{}, sp{}, ep{};   // commutator, Toeplitz, sheared, E^T planes
  float* xsh = nullptr;    // exchange sums, un-sheared: 3 x Nw x Nk x Nk complex (FP32)
  void* block = nullptr;   // one allocation for the per-wire vectors below
  int* ints = nullptr;     // eS, eH, eT, eE, esc, esx, ess, (spare), eO  (9 x nw)
  unsigned* mx = nullptr;  // Hamiltonian, state, hbar A/B and off-diagonal maxima (4 x nw)
  unsigned long long* mx64 = nullptr;   // nw: FP64 maxima of the phonon tables
  float* vsf = nullptr;    // 3 x nw x nk screened V by |k1 - k2|
  float2* trf = nullptr;   // 4 x nw x nk traces [2][2nk]
  float* gamf = nullptr;   // 2 x nw x nk GamE, GamH
  float2* dgf = nullptr;   // 4 x nw x nk: hi and lo parts of the peeled Hee, Hhh diagonals
  double2 *dgE = nullptr, *dgH = nullptr;  // the peeled diagonals in FP64
  float* xef = nullptr;     // 2 x nw x nk |xe|, |xh|
  int* sP = nullptr;        // nw phonon-table exponents
  float* phf = nullptr;     // 2 x nw x nk: Vep(d) 2^-sP, Vhp(d) 2^-sP
  float* gtab = nullptr;    // 4 x nw x nk: gamma weights per q
  float2* tpart = nullptr;  // nw x 2 x 32 ceil(2nk/32) x T diagonal partials (T = ceil(nk/32))
  float* cdf = nullptr;     // 4 x nw x nk: hi / lo parts of Re C_kk and Re D_kk (stage state)
  double* xdg = nullptr;    // 2 x nw x nk: Re C_kk, Re D_kk of the stage state in FP64
  int* eS() { return ints; }
  int* eH() { return ints + nw; }
  int* eT() { return ints + 2 * nw; }
  int* eE() { return ints + 3 * nw; }
  int* esc() { return ints + 4 * nw; }
  int* esx() { return ints + 5 * nw; }
  int* ess() { return ints + 6 * nw; }
  int* eO() { return ints + 8 * nw; }   // commutator state operands (diagonals of C, D peeled)
  unsigned* mxH() { return mx; }
  unsigned* mxS() { return mx + nw; }
  unsigned* mxAB() { return mx + 2 * nw; }
  unsigned* mxO() { return mx + 3 * nw; }  // max over P and the off-diagonal C, D
};

struct MixedAll {
  std::vector<Mixed*> b;     // buckets by ascending Nk
  void* block = nullptr;     // the context-wide FP32 buffers
  float2* kf = nullptr;      // 3 x tot_mat stage derivatives
  float2* accf = nullptr;    // 3 x tot_mat RK4 sums k1 + 2 k2 + 2 k3
  float2* hf = nullptr;      // 3 x tot_mat Heh, Hee', Hhh'
  float* habf = nullptr;     // 2 x tot_mat hbar A, hbar B
  float* epf = nullptr;      // EP, EP^T, HP, HP^T scaled by 2^sP (tot_mat each)
  float *eptf = nullptr, *hpf = nullptr, *hptf = nullptr;
  float2* ekf = nullptr;     // 3 x tot_r stage field
  float2* ekrf = nullptr;    // tot_kr Expikr
  int* err = nullptr;        // engine error flag (bounded waits that gave up)
};

// matrix slots of the commutator plane sets
enum { M_P = 0, M_PT, M_C, M_CT, M_D, M_DT, M_EH, M_EHT, M_EE, M_EET, M_HH, M_HHT, M_EEX, M_HHX };

static inline MixedAll* all_of(SbeCtx* c) { return static_cast<MixedAll*>(c->mixed); }

// GEMM kinds of a stage: exchange products (real), commutators (dP with the cross
// terms of W and V), hi*hi products of W and V, sources
// Slots of the context's G buffer (tot_mat FP32 complex each, indexed like the
// packed state) that one stage's commutator GEMMs write: W, V (cross terms from the dP
// launch, hi*hi parts added by the hi*hi launch) and the dP sums
enum GSlot : int { G_W = 0, G_V = 1, G_DP = 2 };

enum JobKind { JK_EXCH = 0, JK_FULL = 1, JK_HH = 2, JK_SRC = 3 };

// The GEMM jobs of one kind for bucket m (its tile choice included).
void bucket_jobs(SbeCtx* c, Mixed* m, int kind, std::vector<tc::GemmJob>& out);
// Launch a job list: consecutive jobs of one N tile share a persistent launch
// (tc::MAX_JOBS per launch).
int launch_jobs(const std::vector<tc::GemmJob>& jobs, cudaStream_t s);

}  // namespace sbe
