// Host-side context of libsbe_gb300: per-wire descriptors and the device arena.
#pragma once
#include <vector>
#include <functional>

#include "sbe_internal.cuh"

struct SbeCtx {
  int nw = 0;
  int nk_max = 0, nr_max = 0;
  std::vector<SbeWireDesc> desc;
  std::vector<sbe::WireDev> wires;  // host copy of d_wires (the caller's wire order)
  std::vector<int> order;           // wires in packed-layout order (grouped by Nk)
  sbe::WireDev* d_wires = nullptr;
  long long tot_mat = 0, tot_vec = 0, tot_r = 0, tot_dd = 0, tot_kr = 0;

  // one arena for everything the context owns
  void* arena = nullptr;
  size_t arena_bytes = 0;

  // ---- tables (FP64, built once) ----
  double *kr = nullptr, *r = nullptr, *Ee = nullptr, *Eh = nullptr;  // vec, r, vec, vec
  double* v0 = nullptr;       // 3*tot_vec: per wire [3][nk] (eh, ee, hh) by k1-k2 >= 0
  double* chi = nullptr;      // 2*tot_vec: per wire [2][nk] Chi1De/Chi1Dh by |k1-k2|
  double* qeh = nullptr;      // 2*tot_vec: per wire [2][nk] qe/qh by |k1-k2|
  int* iq = nullptr;          // tot_vec: round(|ky/dq|) of Vxx2
  double *EP = nullptr, *HP = nullptr;  // tot_mat
  int* maps = nullptr;        // 6*tot_mat: k_p_q, k_m_q, k1p, k1p_m_q, k1, k1_m_q
  double* xeh = nullptr;      // 2*tot_vec
  double* window = nullptr;   // tot_r
  double2* expikr = nullptr;  // tot_kr  [nk][nr]
  double2* wk = nullptr;      // tot_r: FFTG(window)
  double* vcorr = nullptr;    // 3*(tot_r + 2*nw): Vint correlation scratch

  // ---- per-step workspace ----
  double2 *ne = nullptr, *nh = nullptr;  // tot_vec
  double* eps = nullptr;                 // tot_vec
  double* vs = nullptr;                  // 3*tot_vec screened V by k1-k2
  double *gamE = nullptr, *gamH = nullptr;
  double *De = nullptr, *Dh = nullptr;   // tot_dd
  double2 *dA = nullptr, *dB = nullptr;  // tot_mat dephasing contraction matrices (real values)
  double2 *Heh = nullptr, *Hee = nullptr, *Hhh = nullptr;  // tot_mat
  double2* tr = nullptr;                 // 4*tot_vec diagonal traces (C, D) per wire [2][2nk]
  double2 *dP = nullptr, *dC = nullptr, *dD = nullptr;     // tot_mat
  double* wrate = nullptr;               // 4*tot_vec Win/Wout e/h
  double* rsp = nullptr;                 // tot_vec spontaneous emission rates (Recomb)
  double2* dcs = nullptr;                // tot_vec DC transport shift kernel s(m) per wire
  double* emis = nullptr;                // emission tables (per wire emis_nw values)
  double2* G = nullptr;                  // 3*tot_kr source GEMM outputs
  double2* qscr = nullptr;               // 20*nr_max + 1: Prop2QW / QW2Prop wire-grid scratch
  double2* p2q_coef = nullptr;           // Prop2QW spline coefficients of the caller's grid
  long long p2q_cap = 0;                 // (12 per grid point; grown on a larger grid)
  double2* kacc = nullptr;               // 3*tot_mat RK4 accumulator
  double2* xs = nullptr;                 // 3*tot_mat RK4 stage state
  double* scal = nullptr;                // 16*nw per-wire scalars
  double* charge = nullptr;              // 2*nw sum |C_kk|, sum |D_kk| before the last normalisation
  double2* ekst = nullptr;               // 3*tot_r stage field
  float* occf = nullptr;                 // 2*tot_vec |ne|, |nh| in FP32
  float* dconst = nullptr;               // 16*nw FP32 dephasing constants
  float* dpre = nullptr;                 // 4*tot_vec FP32 dephasing prefactors per |q|

  int* dwl = nullptr;                    // nw wire indices, grouped (dephasing groups)
  // groups of wires with identical dephasing constants (Nk, masses, grid, rates):
  // (first index into dwl, count)
  std::vector<std::pair<int, int>> dgroups;
  std::vector<int> dwl_host;              // host copy of dwl

  int any_offdiag = 0;                   // some wire has OffDiagDph on
  void* mixed = nullptr;                 // mixed-precision workspace (sbe_tc.cu)

  // kernel timing (sbe_ctx_profile): event pairs per category, and a pool
  int prof = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_ev[4];
  std::vector<cudaEvent_t> ev_pool;
};

namespace sbe {
// Records a pair of events around the launches in its scope when profiling is on.
struct ProfScope {
  SbeCtx* c;
  int cat;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  static cudaEvent_t take(SbeCtx* c) {
    cudaEvent_t e;
    if (!c->ev_pool.empty()) {
      e = c->ev_pool.back();
      c->ev_pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  }
  ProfScope(SbeCtx* c_, int cat_, cudaStream_t s_) : c(c_), cat(cat_), s(s_) {
    if (c->prof) {
      a = take(c);
      b = take(c);
      cudaEventRecord(a, s);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEventRecord(b, s);
      c->prof_ev[cat].push_back({a, b});
    }
  }
};
int mixed_prepare(SbeCtx* c, cudaStream_t s);
int tc_gemm_init();
}  // namespace sbe

namespace sbe {
// sbe_tables.cu
int build_tables(SbeCtx* c, cudaStream_t s);
// sbe_prep.cu
void launch_prep_scalar(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s);
void launch_expand_vc(SbeCtx* c, int w, double* VC, double* E1D, cudaStream_t s);
void launch_gamma(SbeCtx* c, int w_only, cudaStream_t s);
void launch_offdiag_D(SbeCtx* c, int w_only, const double* g3, bool fp32, cudaStream_t s);
void launch_offdiag_AB(SbeCtx* c, int w_only, cudaStream_t s);
void launch_traces(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s);
void launch_calch_ctx(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                      const double2* Ek, cudaStream_t s);
int launch_calch_single(int nk, const double2* Meh, const double2* Wee, const double2* Whh,
                        const double2* C, const double2* D, const double2* P, const double* VC,
                        const double* Ee, const double* Eh, double gap, int excitons, int lf,
                        int freepot, double2* Heh, double2* Hee, double2* Hhh, cudaStream_t s);
// sbe_gemm64.cu
enum Op { OP_N = 0, OP_T = 1, OP_C = 2, OP_H = 3 };
struct Term {
  const void* A;
  const void* B;
  int opA, opB;
  int realA;        // A is a real (double) matrix
  double2 alpha;
};
struct GemmBatch {
  int nterms;
  Term t[6];
  double2* out;
  int epi;          // 0 none, 1 dP epilogue
  // dP epilogue inputs
  const double2* Heh;
  const double2* P;
  const double* gamE;
  const double* gamH;
  const double2* offp;  // optional explicit OffP (single-wire API)
  int w_only = -1;      // >= 0: only this wire of the context
  int flag_mask = 0;    // != 0: only the wires whose flags hold every bit of it (batched)
};
void launch_gemm64(const WireDev* d_wires, int nw, int nk_max, const GemmBatch& b,
                   bool batched, int nk_single, cudaStream_t s);
void launch_sources_gemm64(SbeCtx* c, const GemmBatch& b, cudaStream_t s);
void launch_rhs64_ctx(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                      double2* dP, double2* dC, double2* dD, cudaStream_t s);
// sbe_step.cu
void launch_leapfrog(SbeCtx* c, double2* const* st9, const double2* Ek, double dt,
                     cudaStream_t s);
// relaxation (rates in wrate, Recomb decay), DC transport of P, C, D (SBE_F_DCTRANS,
// field Ek at q = 0) and charge normalisation, in the reference's order
void launch_relax_norm(SbeCtx* c, double2* P3, double2* C3, double2* D3, const double2* Ek,
                       double dt, cudaStream_t s);
void launch_sources(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                    const double2* ne, const double2* nh, double2* src, cudaStream_t s,
                    int w_only = -1);
void launch_extract_diag(SbeCtx* c, const double2* C, const double2* D, cudaStream_t s);
void launch_screen(SbeCtx* c, int w_only, cudaStream_t s);
void launch_phonon_rates_one(SbeCtx* c, int w, cudaStream_t s);
// sbe_emission.cu: spontaneous emission rates (Recomb) of the prepared occupations
void launch_spont(SbeCtx* c, int w_only, cudaStream_t s);
// the InitializeEmission table of one wire (host, FP64): nw values, spacing dhw
std::vector<double> emission_table(const WireDev& W, int* nw, double* dhw);
// sbe_mbc.cu: carrier-carrier scattering rates (EHs) added to wrate
void launch_mbc_rates(SbeCtx* c, int w_only, cudaStream_t s, bool all = false,
                      bool fp32 = false);
void launch_leap_shuffle(SbeCtx* c, double2* const* st, cudaStream_t s);
void add_rates(const double* wrate, int nk, double* a, double* b, double* cc, double* d,
               cudaStream_t s);
// sbe_tc.cu (mixed precision)
void mixed_free(SbeCtx* c);
int rhs_mixed(SbeCtx* c, const double2* P, const double2* C, const double2* D, const double2* Ek,
              double2* dP, double2* dC, double2* dD, cudaStream_t s);
void launch_sources_reduce(SbeCtx* c, const double2* ne, const double2* nh, double2* src,
                           cudaStream_t s);
void launch_sources_final(SbeCtx* c, const double2* ne, const double2* nh, double2* src,
                          cudaStream_t s);
void launch_relax_only(SbeCtx* c, double2* P3, double2* C3, double2* D3, const double2* Ek,
                       double dt, cudaStream_t s);
// sbe_info.cu: per-step statistics of wire w (info / EP columns) into out (23 doubles)
int launch_wire_info(SbeCtx* c, int w, const double2* C2, const double2* D2, const double2* src,
                     const double2* Ek, double* out, cudaStream_t s);
// sbe_info.cu: wire-grid P.E increment (PdotE.w.dat) and the De / Dh extrema
// (MaxOffDiag.{e,h}.dat) of wire w
int launch_wire_pdote(SbeCtx* c, int w, const double2* Ek, const double2* src, const double* P0,
                      double* out, cudaStream_t s);
int launch_deph_extrema(SbeCtx* c, int w, double* out4, cudaStream_t s);
// sbe_dc.cu: DC transport (dcfield.py:1154-1236 Transport) of P, C, D
bool any_dc(const SbeCtx* c);
void launch_dc_transport(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek,
                         double dt, cudaStream_t s);
int rk4_mixed(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek0,
              const double2* dEk, double dt, double2* src, cudaStream_t s);
void launch_rk4_axpy(SbeCtx* c, int stage, double dt, double2* P, double2* C, double2* D,
                     cudaStream_t s);
void launch_stage_field(SbeCtx* c, const double2* Ek0, const double2* dEk, double frac,
                        cudaStream_t s);
int launch_prop2qw(SbeCtx* c, int w, const double* RR, int n_rr, const double2* fin,
                   double2* out, cudaStream_t s);
int launch_prop2qw_scratch(SbeCtx* c, int w, const double* RR, int n_rr, const double2* fin,
                           double2* out, double2* coef, double2* tmp, cudaStream_t s);
int capture_graph(SbeCtx* c, int precision, const std::function<int(cudaStream_t)>& body,
                  SbeGraph** out, long long* n_kernels);
int launch_qw2prop(SbeCtx* c, int w, const double* RR, int n_rr, const double2* src,
                   double2* out, int plasmonics, cudaStream_t s);
}  // namespace sbe
