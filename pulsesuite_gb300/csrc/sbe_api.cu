// C ABI of libsbe_gb300: context management and the entry points declared in
// include/sbe_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "sbe_ctx.cuh"

namespace sbe {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SBE_OK;
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return SBE_ERR_CUDA;
}

// Host copy of derived constants: SBEs.py:4794-4823, phonons.py:104-136.
static WireDev derive(const SbeWireDesc& d, int nk_check_only = 0) {
  (void)nk_check_only;
  WireDev W{};
  W.nk = d.nk;
  W.nr = 2 * d.nk + 2;
  W.flags = d.flags;
  W.w = d.wire_index;
  W.yw = ((int)std::floor((d.wire_index - 1) / 2.0) % 2 == 0) ? 1 : -1;
  W.zsign = (d.wire_index % 2 == 0) ? 1 : -1;
  W.dnk = (d.nk - 1) / 2;
  W.L = d.L;
  W.dkr = kTwoPi / (2.0 * d.L);
  W.Delta0 = d.Delta0;
  W.gap = d.gap;
  W.me = d.me;
  W.mh = d.mh;
  W.HO = d.HO;
  W.gam_e = d.gam_e;
  W.gam_h = d.gam_h;
  W.gam_eh = d.gam_eh;
  W.epsr = d.epsr;
  W.Oph = d.Oph;
  W.Gph = d.Gph;
  W.temp = d.temp;
  W.Edc = d.Edc;
  W.dcv = std::sqrt((kE0 * kHbar) * (kE0 * kHbar) / (6.0 * kMe0 * d.gap) * (kMe0 / d.me - 1.0));
  W.alphae = std::sqrt(d.me * d.HO) / kHbar;
  W.alphah = std::sqrt(d.mh * d.HO) / kHbar;
  double ae = W.alphae, ah = W.alphah;
  W.ehint = std::sqrt(2.0 * ae * ah / (ae * ae + ah * ah));
  W.qc = 2.0 * ae * ah / (ae + ah);
  W.area = std::sqrt(2.0 * kPi) / std::sqrt(ae * ae + ah * ah) * d.Delta0;
  W.vscale = kHbar * d.Oph * d.epsr * (1.0 / 8.2 - 1.0 / 10.0);
  W.n0ph = 1.0 / (std::exp(kHbar * d.Oph / kKb / d.temp) - 1.0);
  W.nmax = std::min(ae / 2.0, ah / 2.0) / kPi * 0.99;
  W.pol_scale = 2.0 * W.ehint / W.area / W.L;
  W.rho_scale = 2.0 * kE0 * W.ehint / W.area;
  const float ed = (float)(W.ehint * W.dcv);
  W.ed_x = ed;
  W.ed_y = -ed * (float)W.yw;
  W.ed_z = ed * (float)W.zsign;
  return W;
}

}  // namespace sbe

using namespace sbe;

extern "C" {

const char* sbe_last_error(void) { return g_err.c_str(); }

int sbe_version(void) { return 1; }

int sbe_constants(double* out5) {
  if (!out5) return fail(SBE_ERR_ARG, "sbe_constants: null output");
  out5[0] = kHbar;
  out5[1] = kE0;
  out5[2] = kEps0;
  out5[3] = kMe0;
  out5[4] = kKb;
  return SBE_OK;
}

static const int kUnsupportedFlags = SBE_F_FREEPOT;

int sbe_ctx_create(const SbeWireDesc* wires, int n_wires, void* stream, SbeCtx** out) {
  if (!wires || n_wires <= 0 || !out) return fail(SBE_ERR_ARG, "sbe_ctx_create: bad arguments");
  *out = nullptr;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return fail(SBE_ERR_CUDA, "sbe_ctx_create: no CUDA device");
  SbeCtx* c = new SbeCtx();
  c->nw = n_wires;
  c->desc.assign(wires, wires + n_wires);
  for (int w = 0; w < n_wires; ++w) {
    const SbeWireDesc& d = wires[w];
    if (d.nk < 4 || d.nk > 4096 || !(d.L > 0) || !(d.me > 0) || !(d.mh > 0) || !(d.HO > 0) ||
        !(d.gap > 0) || !(d.Delta0 > 0) || !(d.epsr > 0) || !(d.temp > 0) || d.wire_index < 1) {
      delete c;
      return fail(SBE_ERR_ARG, "sbe_ctx_create: invalid wire descriptor " + std::to_string(w));
    }
    if (d.flags & kUnsupportedFlags) {
      delete c;
      return fail(SBE_ERR_UNSUPPORTED,
                  "sbe_ctx_create: FreePot is not built (wire " +
                      std::to_string(w) + ")");
    }
    WireDev W = derive(d);
    W.off_tab = w;
    c->nk_max = std::max(c->nk_max, W.nk);
    c->nr_max = std::max(c->nr_max, W.nr);
    if (d.flags & SBE_F_OFFDIAGDPH) c->any_offdiag = 1;
    c->wires.push_back(W);
  }
  // packed layout: wires grouped by Nk (ascending, stable), so that the wires of one
  // Nk are one contiguous block of every packed buffer (the mixed path's buckets);
  // a context of one Nk keeps the order of its wires
  c->order.resize(n_wires);
  for (int w = 0; w < n_wires; ++w) c->order[w] = w;
  std::stable_sort(c->order.begin(), c->order.end(),
                   [&](int a, int b) { return c->wires[a].nk < c->wires[b].nk; });
  long long om = 0, ov = 0, orr = 0, odd = 0, okr = 0;
  for (int w : c->order) {
    WireDev& W = c->wires[w];
    W.off_mat = om;
    W.off_vec = ov;
    W.off_r = orr;
    W.off_dd = odd;
    W.off_kr = okr;
    om += (long long)W.nk * W.nk;
    ov += W.nk;
    orr += W.nr;
    odd += (long long)(2 * W.nk + 1) * W.nk;
    okr += (long long)W.nk * W.nr;
  }
  c->tot_mat = om;
  c->tot_vec = ov;
  c->tot_r = orr;
  c->tot_dd = odd;
  c->tot_kr = okr;

  // arena layout
  struct Part { void** p; size_t bytes; };
  std::vector<Part> parts;
  auto add = [&](void** p, size_t bytes) { parts.push_back({p, bytes}); };
  const size_t D8 = 8, C16 = 16;
  add((void**)&c->kr, D8 * ov);
  add((void**)&c->r, D8 * orr);
  add((void**)&c->Ee, D8 * ov);
  add((void**)&c->Eh, D8 * ov);
  add((void**)&c->v0, D8 * 3 * ov);
  add((void**)&c->chi, D8 * 2 * ov);
  add((void**)&c->qeh, D8 * 2 * ov);
  add((void**)&c->iq, 4 * ov);
  add((void**)&c->EP, D8 * om);
  add((void**)&c->HP, D8 * om);
  add((void**)&c->maps, 4 * 6 * om);
  add((void**)&c->xeh, D8 * 2 * ov);
  add((void**)&c->window, D8 * orr);
  add((void**)&c->expikr, C16 * okr);
  add((void**)&c->wk, C16 * orr);
  add((void**)&c->vcorr, D8 * 3 * (orr + 2 * n_wires));
  add((void**)&c->ne, C16 * ov);
  add((void**)&c->nh, C16 * ov);
  add((void**)&c->eps, D8 * ov);
  add((void**)&c->vs, D8 * 3 * ov);
  add((void**)&c->gamE, D8 * ov);
  add((void**)&c->gamH, D8 * ov);
  add((void**)&c->De, D8 * odd);
  add((void**)&c->Dh, D8 * odd);
  add((void**)&c->dA, C16 * om);
  add((void**)&c->dB, C16 * om);
  add((void**)&c->Heh, C16 * om);
  add((void**)&c->Hee, C16 * om);
  add((void**)&c->Hhh, C16 * om);
  add((void**)&c->tr, C16 * 4 * ov);
  add((void**)&c->dP, C16 * om);
  add((void**)&c->dC, C16 * om);
  add((void**)&c->dD, C16 * om);
  add((void**)&c->wrate, D8 * 4 * ov);
  add((void**)&c->rsp, D8 * ov);
  add((void**)&c->dcs, C16 * ov);
  // emission tables (Recomb): InitializeEmission on the host, per wire
  std::vector<double> emis_host;
  for (auto& W : c->wires) {
    W.emis_nw = 0;
    W.emis_dhw = 0.0;
    W.off_emis = (long long)emis_host.size();
    if (!(W.flags & SBE_F_RECOMB)) continue;
    int nwv = 0;
    double dhw = 0.0;
    std::vector<double> t = emission_table(W, &nwv, &dhw);
    if (nwv < 10) {
      delete c;
      return fail(SBE_ERR_ARG, "sbe_ctx_create: temperature too low for the emission grid "
                               "(emission.py CalcHOmega)");
    }
    W.emis_nw = nwv;
    W.emis_dhw = dhw;
    emis_host.insert(emis_host.end(), t.begin(), t.end());
  }
  add((void**)&c->emis, D8 * std::max<size_t>(emis_host.size(), 1));
  add((void**)&c->G, C16 * 3 * okr);
  add((void**)&c->qscr, C16 * (20 * (size_t)c->nr_max + 1));
  add((void**)&c->kacc, C16 * 3 * om);
  add((void**)&c->xs, C16 * 3 * om);
  add((void**)&c->scal, D8 * 16 * n_wires);
  add((void**)&c->charge, D8 * 2 * n_wires);
  add((void**)&c->ekst, C16 * 3 * orr);
  add((void**)&c->occf, 4 * 2 * ov);
  add((void**)&c->dconst, 4 * 16 * (size_t)n_wires);
  add((void**)&c->dpre, 4 * 4 * ov);
  add((void**)&c->dwl, sizeof(int) * (size_t)n_wires);
  size_t total = 0;
  for (auto& p : parts) total += (p.bytes + 255) / 256 * 256;
  if (cudaMalloc(&c->arena, total) != cudaSuccess) {
    delete c;
    return fail(SBE_ERR_OOM, "sbe_ctx_create: arena allocation of " + std::to_string(total) +
                                 " bytes failed");
  }
  c->arena_bytes = total;
  char* base = static_cast<char*>(c->arena);
  size_t off = 0;
  for (auto& p : parts) {
    *p.p = base + off;
    off += (p.bytes + 255) / 256 * 256;
  }
  cudaStream_t s = as_stream(stream);
  cudaMemsetAsync(c->arena, 0, total, s);
  if (cudaMalloc(&c->d_wires, sizeof(WireDev) * n_wires) != cudaSuccess) {
    cudaFree(c->arena);
    delete c;
    return fail(SBE_ERR_OOM, "sbe_ctx_create: descriptor allocation failed");
  }
  cudaMemcpyAsync(c->d_wires, c->wires.data(), sizeof(WireDev) * n_wires, cudaMemcpyHostToDevice,
                  s);
  if (!emis_host.empty()) {
    cudaMemcpyAsync(c->emis, emis_host.data(), sizeof(double) * emis_host.size(),
                    cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);   // the host vector is released at the end of this call
  }
  // dephasing groups: wires whose Lorentzian factors coincide (same Nk, masses, grid
  // spacing and broadening rates) share them in the FP32 dephasing sums
  {
    std::vector<int> order;
    std::vector<char> used(n_wires, 0);
    for (int a = 0; a < n_wires; ++a) {
      if (used[a]) continue;
      const WireDev& A = c->wires[a];
      const int first = (int)order.size();
      for (int b = a; b < n_wires; ++b) {
        const WireDev& B = c->wires[b];
        if (used[b] || B.nk != A.nk || B.dnk != A.dnk || B.me != A.me || B.mh != A.mh ||
            B.dkr != A.dkr || B.gam_e != A.gam_e || B.gam_h != A.gam_h || B.gam_eh != A.gam_eh)
          continue;
        used[b] = 1;
        order.push_back(b);
      }
      c->dgroups.emplace_back(first, (int)order.size() - first);
    }
    c->dwl_host = order;
    cudaMemcpyAsync(c->dwl, c->dwl_host.data(), sizeof(int) * n_wires, cudaMemcpyHostToDevice, s);
  }
  int rc = build_tables(c, s);
  if (rc == SBE_OK) rc = cuda_check(cudaStreamSynchronize(s), "sbe_ctx_create: table build");
  if (rc != SBE_OK) {
    cudaFree(c->d_wires);
    cudaFree(c->arena);
    delete c;
    return rc;
  }
  *out = c;
  return SBE_OK;
}

int sbe_ctx_destroy(SbeCtx* c) {
  if (!c) return SBE_OK;
  int rc = SBE_OK;
  for (auto& v : c->prof_ev)
    for (auto& pr : v) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  if (c->d_wires && cudaFree(c->d_wires) != cudaSuccess) rc = SBE_ERR_CUDA;
  if (c->arena && cudaFree(c->arena) != cudaSuccess) rc = SBE_ERR_CUDA;
  if (c->p2q_coef && cudaFree(c->p2q_coef) != cudaSuccess) rc = SBE_ERR_CUDA;
  sbe::mixed_free(c);
  delete c;
  if (rc != SBE_OK) set_error("sbe_ctx_destroy: cudaFree failed");
  return rc;
}

int sbe_ctx_layout(const SbeCtx* c, long long* out, long long* total_mat, long long* total_r) {
  if (!c) return fail(SBE_ERR_ARG, "sbe_ctx_layout: null context");
  for (int w = 0; out && w < c->nw; ++w) {
    out[3 * w + 0] = c->wires[w].nk;
    out[3 * w + 1] = c->wires[w].off_mat;
    out[3 * w + 2] = c->wires[w].off_r;
  }
  if (total_mat) *total_mat = c->tot_mat;
  if (total_r) *total_r = c->tot_r;
  return SBE_OK;
}

int sbe_ctx_table(const SbeCtx* c, int w, int which, void* dst, long long nbytes, void* stream) {
  if (!c || w < 0 || w >= c->nw || !dst) return fail(SBE_ERR_ARG, "sbe_ctx_table: bad arguments");
  const WireDev& W = c->wires[w];
  const void* src = nullptr;
  long long need = 0;
  long long nk = W.nk, nr = W.nr;
  switch (which) {
    case 0: src = c->kr + W.off_vec; need = 8 * nk; break;
    case 1: src = c->r + W.off_r; need = 8 * nr; break;
    case 2: src = c->Ee + W.off_vec; need = 8 * nk; break;
    case 3: src = c->Eh + W.off_vec; need = 8 * nk; break;
    case 4: src = c->v0 + 3 * W.off_vec; need = 8 * 3 * nk; break;
    case 5: src = c->chi + 2 * W.off_vec; need = 8 * 2 * nk; break;
    case 6: src = c->qeh + 2 * W.off_vec; need = 8 * 2 * nk; break;
    case 7: src = c->EP + W.off_mat; need = 8 * nk * nk; break;
    case 8: src = c->HP + W.off_mat; need = 8 * nk * nk; break;
    case 9: src = c->window + W.off_r; need = 8 * nr; break;
    case 10: src = c->maps + 6 * W.off_mat; need = 4 * 6 * nk * nk; break;
    case 11: src = c->xeh + 2 * W.off_vec; need = 8 * 2 * nk; break;
    case 12: src = c->expikr + W.off_kr; need = 16 * nk * nr; break;
    case 13: {
      double sc[16] = {W.dcv, W.alphae, W.alphah, W.ehint, W.area, W.qc, W.vscale, W.n0ph,
                       W.nmax, W.dkr, W.L, 0, 0, 0, 0, 0};
      if (nbytes < (long long)sizeof(sc)) return fail(SBE_ERR_ARG, "sbe_ctx_table: buffer small");
      return cuda_check(cudaMemcpyAsync(dst, sc, sizeof(sc), cudaMemcpyHostToDevice,
                                        as_stream(stream)),
                        "sbe_ctx_table");
    }
    case 14: src = c->wk + W.off_r; need = 16 * nr; break;
    default: return fail(SBE_ERR_ARG, "sbe_ctx_table: unknown table");
  }
  if (nbytes < need) return fail(SBE_ERR_ARG, "sbe_ctx_table: destination too small");
  return cuda_check(cudaMemcpyAsync(dst, src, need, cudaMemcpyDeviceToDevice, as_stream(stream)),
                    "sbe_ctx_table");
}

// ---- single-wire reference functions ---------------------------------------
static int rhs_single(int which, int nk, const double* C, const double* D, const double* P,
                      const double* Heh, const double* Hee, const double* Hhh, const double* GamE,
                      const double* GamH, const double* OffP, double* out, void* stream) {
  if (nk < 1 || !C || !D || !P || !Heh || !Hee || !Hhh || !out)
    return fail(SBE_ERR_ARG, "sbe_rhs single: null pointer or bad nk");
  const double ih = 1.0 / kHbar;
  const double2 pos = make_double2(0.0, -ih), neg = make_double2(0.0, ih);
  auto T = [](const void* A, int oa, const void* B, int ob, double2 al) {
    Term t;
    t.A = A; t.B = B; t.opA = oa; t.opB = ob; t.realA = 0; t.alpha = al;
    return t;
  };
  GemmBatch b{};
  const double2 *c2 = (const double2*)C, *d2 = (const double2*)D, *p2 = (const double2*)P;
  const double2 *heh = (const double2*)Heh, *hee = (const double2*)Hee, *hhh = (const double2*)Hhh;
  if (which == 0) {
    if (!GamE || !GamH) return fail(SBE_ERR_ARG, "sbe_dpdt: null rates");
    b.t[b.nterms++] = T(hhh, OP_N, p2, OP_N, pos);
    b.t[b.nterms++] = T(d2, OP_T, heh, OP_T, neg);
    b.t[b.nterms++] = T(p2, OP_N, hee, OP_T, pos);
    b.t[b.nterms++] = T(heh, OP_T, c2, OP_N, neg);
    b.epi = 1;
    b.Heh = heh;
    b.P = p2;
    b.gamE = GamE;
    b.gamH = GamH;
    b.offp = (const double2*)OffP;
  } else if (which == 1) {
    b.t[b.nterms++] = T(c2, OP_N, hee, OP_T, pos);
    b.t[b.nterms++] = T(hee, OP_T, c2, OP_N, neg);
    b.t[b.nterms++] = T(p2, OP_H, heh, OP_T, pos);
    b.t[b.nterms++] = T(heh, OP_C, p2, OP_N, neg);
  } else {
    b.t[b.nterms++] = T(d2, OP_N, hhh, OP_T, pos);
    b.t[b.nterms++] = T(hhh, OP_T, d2, OP_N, neg);
    b.t[b.nterms++] = T(p2, OP_C, heh, OP_N, pos);
    b.t[b.nterms++] = T(heh, OP_H, p2, OP_T, neg);
  }
  b.out = (double2*)out;
  launch_gemm64(nullptr, 1, nk, b, false, nk, as_stream(stream));
  return cuda_check(cudaGetLastError(), "sbe rhs single");
}

int sbe_dpdt(int nk, const double* C, const double* D, const double* P, const double* Heh,
             const double* Hee, const double* Hhh, const double* GamE, const double* GamH,
             const double* OffP, double* out, void* stream) {
  return rhs_single(0, nk, C, D, P, Heh, Hee, Hhh, GamE, GamH, OffP, out, stream);
}

int sbe_dCdt(int nk, const double* C, const double* D, const double* P, const double* Heh,
             const double* Hee, const double* Hhh, double* out, void* stream) {
  return rhs_single(1, nk, C, D, P, Heh, Hee, Hhh, nullptr, nullptr, nullptr, out, stream);
}

int sbe_dDdt(int nk, const double* C, const double* D, const double* P, const double* Heh,
             const double* Hee, const double* Hhh, double* out, void* stream) {
  return rhs_single(2, nk, C, D, P, Heh, Hee, Hhh, nullptr, nullptr, nullptr, out, stream);
}

int sbe_calch(int nk, const double* Meh, const double* Wee, const double* Whh, const double* C,
              const double* D, const double* P, const double* VC, const double* Ee,
              const double* Eh, double gap, int excitons, int lf, int freepot, double* Heh,
              double* Hee, double* Hhh, void* stream) {
  if (nk < 1 || !Meh || !C || !D || !P || !VC || !Ee || !Eh || !Heh || !Hee || !Hhh ||
      (freepot && (!Wee || !Whh)))
    return fail(SBE_ERR_ARG, "sbe_calch: null pointer or bad nk");
  return launch_calch_single(nk, (const double2*)Meh, (const double2*)Wee, (const double2*)Whh,
                             (const double2*)C, (const double2*)D, (const double2*)P, VC, Ee, Eh,
                             gap, excitons, lf, freepot, (double2*)Heh, (double2*)Hee,
                             (double2*)Hhh, as_stream(stream));
}

// ---- per-wire building blocks ----------------------------------------------
static int check_w(SbeCtx* c, int w, const char* who) {
  if (!c || w < 0 || w >= c->nw) return fail(SBE_ERR_ARG, std::string(who) + ": bad context/wire");
  return SBE_OK;
}

static void copy_in(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s);
}

__global__ void k_vs_from_vc(int nk, const double* VC, const double* E1D, double* vs, double* eps) {
  int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nk) return;
  for (int n = 0; n < 3; ++n) vs[n * nk + d] = VC[((long long)d * nk + 0) * 3 + n];
  if (E1D) eps[d] = E1D[(long long)d * nk + 0];
}

static void set_vc(SbeCtx* c, int w, const double* VC, const double* E1D, cudaStream_t s) {
  const WireDev& W = c->wires[w];
  k_vs_from_vc<<<(W.nk + 127) / 128, 128, 0, s>>>(W.nk, VC, E1D, c->vs + 3 * W.off_vec,
                                                  c->eps + W.off_vec);
}

int sbe_screened_arrays(SbeCtx* c, int w, const double* ne, const double* nh, double* VC,
                        double* E1D, void* stream) {
  int rc = check_w(c, w, "sbe_screened_arrays");
  if (rc) return rc;
  if (!ne || !nh || !VC || !E1D) return fail(SBE_ERR_ARG, "sbe_screened_arrays: null pointer");
  cudaStream_t s = as_stream(stream);
  const WireDev& W = c->wires[w];
  copy_in(c->ne + W.off_vec, ne, 16 * W.nk, s);
  copy_in(c->nh + W.off_vec, nh, 16 * W.nk, s);
  launch_screen(c, w, s);
  launch_expand_vc(c, w, VC, E1D, s);
  return cuda_check(cudaGetLastError(), "sbe_screened_arrays");
}

int sbe_gamma(SbeCtx* c, int w, const double* ne, const double* nh, const double* VC,
              double* GamE, double* GamH, void* stream) {
  int rc = check_w(c, w, "sbe_gamma");
  if (rc) return rc;
  if (!ne || !nh || !VC || !GamE || !GamH) return fail(SBE_ERR_ARG, "sbe_gamma: null pointer");
  cudaStream_t s = as_stream(stream);
  const WireDev& W = c->wires[w];
  copy_in(c->ne + W.off_vec, ne, 16 * W.nk, s);
  copy_in(c->nh + W.off_vec, nh, 16 * W.nk, s);
  set_vc(c, w, VC, nullptr, s);
  launch_gamma(c, w, s);
  copy_in(GamE, c->gamE + W.off_vec, 8 * W.nk, s);
  copy_in(GamH, c->gamH + W.off_vec, 8 * W.nk, s);
  return cuda_check(cudaGetLastError(), "sbe_gamma");
}

int sbe_offdiag(SbeCtx* c, int w, const double* ne, const double* nh, const double* P,
                const double* VC, const double* g3, double* x, double* De, double* Dh,
                void* stream) {
  int rc = check_w(c, w, "sbe_offdiag");
  if (rc) return rc;
  if (!ne || !nh || !P || !VC || !g3 || !x) return fail(SBE_ERR_ARG, "sbe_offdiag: null pointer");
  cudaStream_t s = as_stream(stream);
  const WireDev& W = c->wires[w];
  double g[3];
  cudaMemcpyAsync(g, g3, sizeof(g), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  copy_in(c->ne + W.off_vec, ne, 16 * W.nk, s);
  copy_in(c->nh + W.off_vec, nh, 16 * W.nk, s);
  set_vc(c, w, VC, nullptr, s);
  launch_offdiag_D(c, w, g, false, s);
  launch_offdiag_AB(c, w, s);
  copy_in(c->xs + W.off_mat, P, 16 * (size_t)W.nk * W.nk, s);
  const double2 ihb = make_double2(0.0, kHbar);
  GemmBatch b{};
  b.w_only = w;
  b.t[0] = Term{c->dA, c->xs, OP_N, OP_N, 0, ihb};
  b.t[1] = Term{c->xs, c->dB, OP_N, OP_T, 0, ihb};
  b.nterms = 2;
  b.out = c->dP;
  b.epi = 0;
  launch_gemm64(c->d_wires, c->nw, c->nk_max, b, true, 0, s);
  copy_in(x, c->dP + W.off_mat, 16 * (size_t)W.nk * W.nk, s);
  size_t ddb = 8 * (size_t)(2 * W.nk + 1) * W.nk;
  if (De) copy_in(De, c->De + W.off_dd, ddb, s);
  if (Dh) copy_in(Dh, c->Dh + W.off_dd, ddb, s);
  return cuda_check(cudaGetLastError(), "sbe_offdiag");
}

int sbe_deph_selftest(SbeCtx* c, const double* C, const double* D, int fp32, double* De,
                      double* Dh, void* stream) {
  if (!c || !C || !D || !De || !Dh) return fail(SBE_ERR_ARG, "sbe_deph_selftest: null pointer");
  cudaStream_t s = as_stream(stream);
  launch_prep_scalar(c, reinterpret_cast<const double2*>(C), reinterpret_cast<const double2*>(D),
                     s);
  launch_offdiag_D(c, -1, nullptr, fp32 != 0, s);
  copy_in(De, c->De, 8 * (size_t)c->tot_dd, s);
  copy_in(Dh, c->Dh, 8 * (size_t)c->tot_dd, s);
  return cuda_check(cudaGetLastError(), "sbe_deph_selftest");
}

int sbe_phonon_rates(SbeCtx* c, int w, const double* ne, const double* nh, const double* VC,
                     const double* E1D, double* WinE, double* WoutE, double* WinH, double* WoutH,
                     void* stream) {
  int rc = check_w(c, w, "sbe_phonon_rates");
  if (rc) return rc;
  if (!ne || !nh || !VC || !E1D || !WinE || !WoutE || !WinH || !WoutH)
    return fail(SBE_ERR_ARG, "sbe_phonon_rates: null pointer");
  cudaStream_t s = as_stream(stream);
  const WireDev& W = c->wires[w];
  copy_in(c->ne + W.off_vec, ne, 16 * W.nk, s);
  copy_in(c->nh + W.off_vec, nh, 16 * W.nk, s);
  set_vc(c, w, VC, E1D, s);
  launch_phonon_rates_one(c, w, s);
  // accumulate into the caller's arrays (MBPE/MBPH add to Win/Wout)
  sbe::add_rates(c->wrate + 4 * W.off_vec, W.nk, WinE, WoutE, WinH, WoutH, s);
  return cuda_check(cudaGetLastError(), "sbe_phonon_rates");
}

int sbe_spont_emission(SbeCtx* c, int w, const double* ne, const double* nh, const double* VC,
                       double* Rsp, void* stream) {
  int rc = check_w(c, w, "sbe_spont_emission");
  if (rc) return rc;
  if (!ne || !nh || !VC || !Rsp) return fail(SBE_ERR_ARG, "sbe_spont_emission: null pointer");
  const WireDev& W = c->wires[w];
  if (!(W.flags & SBE_F_RECOMB))
    return fail(SBE_ERR_ARG, "sbe_spont_emission: the wire was created without Recomb "
                             "(no emission tables)");
  cudaStream_t s = as_stream(stream);
  copy_in(c->ne + W.off_vec, ne, 16 * W.nk, s);
  copy_in(c->nh + W.off_vec, nh, 16 * W.nk, s);
  set_vc(c, w, VC, nullptr, s);
  launch_spont(c, w, s);
  copy_in(Rsp, c->rsp + W.off_vec, 8 * W.nk, s);
  return cuda_check(cudaGetLastError(), "sbe_spont_emission");
}

int sbe_wire_info(SbeCtx* c, int w, const double* C2, const double* D2, const double* src,
                  const double* Ek, const double* VC, double* out23, void* stream) {
  int rc = check_w(c, w, "sbe_wire_info");
  if (rc) return rc;
  if (!C2 || !D2 || !src || !Ek || !out23) return fail(SBE_ERR_ARG, "sbe_wire_info: null pointer");
  cudaStream_t s = as_stream(stream);
  if (VC) set_vc(c, w, VC, nullptr, s);
  return launch_wire_info(c, w, (const double2*)C2, (const double2*)D2, (const double2*)src,
                          (const double2*)Ek, out23, s);
}

int sbe_wire_pdote(SbeCtx* c, int w, const double* Ek, const double* src, const double* P0,
                   double* out, void* stream) {
  int rc = check_w(c, w, "sbe_wire_pdote");
  if (rc) return rc;
  if (!Ek || !src || !out) return fail(SBE_ERR_ARG, "sbe_wire_pdote: null pointer");
  return launch_wire_pdote(c, w, (const double2*)Ek, (const double2*)src, P0, out,
                           as_stream(stream));
}

int sbe_deph_extrema(SbeCtx* c, int w, double* out4, void* stream) {
  int rc = check_w(c, w, "sbe_deph_extrema");
  if (rc) return rc;
  if (!out4) return fail(SBE_ERR_ARG, "sbe_deph_extrema: null pointer");
  return launch_deph_extrema(c, w, out4, as_stream(stream));
}

int sbe_carrier_rates(SbeCtx* c, int w, const double* ne, const double* nh, const double* VC,
                      double* WinE, double* WoutE, double* WinH, double* WoutH, int precision,
                      void* stream) {
  int rc = check_w(c, w, "sbe_carrier_rates");
  if (rc) return rc;
  if (!ne || !nh || !VC || !WinE || !WoutE || !WinH || !WoutH)
    return fail(SBE_ERR_ARG, "sbe_carrier_rates: null pointer");
  if (precision != SBE_PREC_FP64 && precision != SBE_PREC_MIXED)
    return fail(SBE_ERR_ARG, "sbe_carrier_rates: precision must be SBE_PREC_FP64 or SBE_PREC_MIXED");
  cudaStream_t s = as_stream(stream);
  const WireDev& W = c->wires[w];
  copy_in(c->ne + W.off_vec, ne, 16 * W.nk, s);
  copy_in(c->nh + W.off_vec, nh, 16 * W.nk, s);
  set_vc(c, w, VC, nullptr, s);
  cudaMemsetAsync(c->wrate + 4 * W.off_vec, 0, sizeof(double) * 4 * W.nk, s);
  launch_mbc_rates(c, w, s, true, precision == SBE_PREC_MIXED);
  // accumulate into the caller's arrays (MBCE/MBCH add to Win/Wout)
  sbe::add_rates(c->wrate + 4 * W.off_vec, W.nk, WinE, WoutE, WinH, WoutH, s);
  return cuda_check(cudaGetLastError(), "sbe_carrier_rates");
}

int sbe_sources(SbeCtx* c, int w, const double* P, const double* C, const double* D,
                const double* ne, const double* nh, double* Px, double* Py, double* Pz,
                double* re, double* rh, void* stream) {
  int rc = check_w(c, w, "sbe_sources");
  if (rc) return rc;
  if (!P || !C || !D || !ne || !nh || !Px || !Py || !Pz || !re || !rh)
    return fail(SBE_ERR_ARG, "sbe_sources: null pointer");
  cudaStream_t s = as_stream(stream);
  const WireDev& W = c->wires[w];
  size_t mb = 16 * (size_t)W.nk * W.nk;
  long long n = c->tot_mat;
  copy_in(c->xs + W.off_mat, P, mb, s);
  copy_in(c->xs + n + W.off_mat, C, mb, s);
  copy_in(c->xs + 2 * n + W.off_mat, D, mb, s);
  copy_in(c->ne + W.off_vec, ne, 16 * W.nk, s);
  copy_in(c->nh + W.off_vec, nh, 16 * W.nk, s);
  double2* src = c->G + 0;  // scratch is the tail of kacc: 5*tot_r <= 3*tot_mat
  src = c->kacc;
  launch_sources(c, c->xs, c->xs + n, c->xs + 2 * n, c->ne, c->nh, src, s, w);
  size_t rb = 16 * (size_t)W.nr;
  const double2* o = src + 5 * W.off_r;
  copy_in(Px, o, rb, s);
  copy_in(Py, o + W.nr, rb, s);
  copy_in(Pz, o + 2 * W.nr, rb, s);
  copy_in(re, o + 3 * W.nr, rb, s);
  copy_in(rh, o + 4 * W.nr, rb, s);
  return cuda_check(cudaGetLastError(), "sbe_sources");
}

int sbe_prop2qw(SbeCtx* c, int w, const double* RR, int n_rr, const double* fields_in,
                double* out, void* stream) {
  int rc = check_w(c, w, "sbe_prop2qw");
  if (rc) return rc;
  if (!RR || n_rr < 2 || !fields_in || !out) return fail(SBE_ERR_ARG, "sbe_prop2qw: bad arguments");
  return launch_prop2qw(c, w, RR, n_rr, (const double2*)fields_in, (double2*)out,
                        as_stream(stream));
}

int sbe_qw2prop(SbeCtx* c, int w, const double* RR, int n_rr, const double* src_in, double* out,
                int plasmonics, void* stream) {
  int rc = check_w(c, w, "sbe_qw2prop");
  if (rc) return rc;
  if (!RR || n_rr < 2 || !src_in || !out) return fail(SBE_ERR_ARG, "sbe_qw2prop: bad arguments");
  return launch_qw2prop(c, w, RR, n_rr, (const double2*)src_in, (double2*)out, plasmonics,
                        as_stream(stream));
}

// ---- whole-context steps ---------------------------------------------------
static void prep_frozen(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                        cudaStream_t s) {
  (void)P;
  launch_prep_scalar(c, C, D, s);
  launch_gamma(c, -1, s);
  if (c->any_offdiag) {
    launch_offdiag_D(c, -1, nullptr, false, s);
    launch_offdiag_AB(c, -1, s);
  }
}

int sbe_rhs(SbeCtx* c, const double* P, const double* C, const double* D, const double* Ek,
            int precision, double* dP, double* dC, double* dD, void* stream) {
  if (!c || !P || !C || !D || !Ek || !dP || !dC || !dD) return fail(SBE_ERR_ARG, "sbe_rhs: null");
  cudaStream_t s = as_stream(stream);
  const double2 *p = (const double2*)P, *cc = (const double2*)C, *d = (const double2*)D;
  if (precision == SBE_PREC_FP64) {
    prep_frozen(c, p, cc, d, s);
    launch_calch_ctx(c, p, cc, d, (const double2*)Ek, s);
    launch_rhs64_ctx(c, p, cc, d, (double2*)dP, (double2*)dC, (double2*)dD, s);
  } else if (precision == SBE_PREC_MIXED) {
    int rc = sbe::rhs_mixed(c, p, cc, d, (const double2*)Ek, (double2*)dP, (double2*)dC,
                            (double2*)dD, s);
    if (rc) return rc;
  } else {
    return fail(SBE_ERR_ARG, "sbe_rhs: unknown precision");
  }
  return cuda_check(cudaGetLastError(), "sbe_rhs");
}

int sbe_leapfrog_step(SbeCtx* c, double* const* state9, const double* Ek, double dt,
                      double* src_out, void* stream) {
  if (!c || !state9 || !Ek || !src_out) return fail(SBE_ERR_ARG, "sbe_leapfrog_step: null");
  for (int i = 0; i < 9; ++i)
    if (!state9[i]) return fail(SBE_ERR_ARG, "sbe_leapfrog_step: null state level");
  cudaStream_t s = as_stream(stream);
  double2* st[9];
  for (int i = 0; i < 9; ++i) st[i] = (double2*)state9[i];
  // SBEs.py:5061-5068: p2 = YY3, C2 = CC3, D2 = DD3 (level 3 is "current")
  prep_frozen(c, st[2], st[5], st[8], s);
  launch_calch_ctx(c, st[2], st[5], st[8], (const double2*)Ek, s);
  launch_rhs64_ctx(c, st[2], st[5], st[8], c->dP, c->dC, c->dD, s);
  launch_leapfrog(c, st, (const double2*)Ek, dt, s);
  launch_sources(c, st[0], st[3], st[6], c->ne, c->nh, (double2*)src_out, s);
  launch_leap_shuffle(c, st, s);
  return cuda_check(cudaGetLastError(), "sbe_leapfrog_step");
}

int sbe_rk4_step(SbeCtx* c, double* P, double* C, double* D, const double* Ek0, const double* dEk,
                 double dt, int precision, double* src_out, void* stream) {
  if (!c || !P || !C || !D || !Ek0 || !src_out) return fail(SBE_ERR_ARG, "sbe_rk4_step: null");
  if (precision == SBE_PREC_MIXED) {
    return sbe::rk4_mixed(c, (double2*)P, (double2*)C, (double2*)D, (const double2*)Ek0,
                         (const double2*)dEk, dt, (double2*)src_out, as_stream(stream));
  }
  if (precision != SBE_PREC_FP64) return fail(SBE_ERR_ARG, "sbe_rk4_step: unknown precision");
  cudaStream_t s = as_stream(stream);
  double2 *p = (double2*)P, *cc = (double2*)C, *d = (double2*)D;
  long long n = c->tot_mat;
  prep_frozen(c, p, cc, d, s);
  const double frac[4] = {0.0, 0.5, 0.5, 1.0};
  for (int st = 1; st <= 4; ++st) {
    const double2 *xp = p, *xc = cc, *xd = d;
    if (st > 1) {
      xp = c->xs;
      xc = c->xs + n;
      xd = c->xs + 2 * n;
    }
    launch_stage_field(c, (const double2*)Ek0, (const double2*)dEk, frac[st - 1], s);
    launch_calch_ctx(c, xp, xc, xd, c->ekst, s);
    launch_rhs64_ctx(c, xp, xc, xd, c->dP, c->dC, c->dD, s);
    launch_rk4_axpy(c, st, dt, p, cc, d, s);
  }
  launch_relax_norm(c, p, cc, d, (const double2*)Ek0, dt, s);
  launch_sources(c, p, cc, d, c->ne, c->nh, (double2*)src_out, s);
  return cuda_check(cudaGetLastError(), "sbe_rk4_step");
}

// ---- local field ---------------------------------------------------------------
// A field uniform along every wire (the local-field drivers, sbetestprop.py:184-198)
// in wire k space: Prop2QW of a constant E is E FFTG(window) (qwoptics.py:667-715 with
// the spline of a constant), so component comp of wire w is e0[w] wk[w] and the
// other two are 0; dEk likewise from de.  One thread per (r, component, wire).
__global__ void k_local_field(const WireDev* wires, const double2* wk, const double* e0,
                              const double* de, int comp, double2* Ek0, double2* dEk) {
  const WireDev W = wires[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * W.nr) return;
  const int f = i / W.nr, r = i - f * W.nr;
  const double2 v = f == comp ? wk[W.off_r + r] : make_double2(0.0, 0.0);
  const long long o = 3 * W.off_r + i;
  const double a = e0[blockIdx.y];
  Ek0[o] = make_double2(a * v.x, a * v.y);
  if (dEk) {
    const double b = de[blockIdx.y];
    dEk[o] = make_double2(b * v.x, b * v.y);
  }
}

int sbe_local_field(SbeCtx* c, const double* e0, const double* de, int comp, double* Ek0,
                    double* dEk, void* stream) {
  if (!c || !e0 || !Ek0 || (dEk && !de) || comp < 0 || comp > 2)
    return fail(SBE_ERR_ARG, "sbe_local_field: bad arguments");
  k_local_field<<<dim3((3 * c->nr_max + 127) / 128, c->nw), 128, 0, as_stream(stream)>>>(
      c->d_wires, c->wk, e0, de, comp, (double2*)Ek0, (double2*)dEk);
  return cuda_check(cudaGetLastError(), "sbe_local_field");
}

// ---- CUDA graph of one step -------------------------------------------------
struct SbeGraph {
  cudaGraphExec_t exec = nullptr;
};

}  // extern "C"

namespace sbe {
// Runs body once on a private non-blocking stream under capture and instantiates
// the graph.  The mixed workspace is prepared (allocated) before the capture.
int capture_graph(SbeCtx* c, int precision, const std::function<int(cudaStream_t)>& body,
                  SbeGraph** out, long long* n_kernels) {
  *out = nullptr;
  if (c->prof) return fail(SBE_ERR_ARG, "graph capture: disable profiling first");
  cudaStream_t cs;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
    return fail(SBE_ERR_CUDA, "graph capture: stream");
  int rc = SBE_OK;
  if (precision == SBE_PREC_MIXED) rc = mixed_prepare(c, cs);
  if (rc == SBE_OK) rc = cuda_check(cudaStreamSynchronize(cs), "graph warm-up");
  cudaGraph_t g = nullptr;
  if (rc == SBE_OK) {
    rc = cuda_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (rc == SBE_OK) {
      int rc2 = body(cs);
      rc = cuda_check(cudaStreamEndCapture(cs, &g), "end capture");
      if (rc2) rc = rc2;
    }
  }
  SbeGraph* sg = nullptr;
  if (rc == SBE_OK) {
    size_t n = 0;
    cudaGraphGetNodes(g, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    cudaGraphGetNodes(g, nodes.data(), &n);
    long long kc = 0;
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kc;
    }
    if (n_kernels) *n_kernels = kc;
    sg = new SbeGraph();
    rc = cuda_check(cudaGraphInstantiate(&sg->exec, g, 0), "graph instantiate");
    if (rc) {
      delete sg;
      sg = nullptr;
    }
  }
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  *out = sg;
  return rc;
}
}  // namespace sbe

extern "C" {

int sbe_rk4_graph_create(SbeCtx* c, double* P, double* C, double* D, const double* Ek0,
                         const double* dEk, double dt, int precision, double* src_out,
                         SbeGraph** out, long long* n_kernels) {
  if (!c || !out) return fail(SBE_ERR_ARG, "sbe_rk4_graph_create: null");
  return sbe::capture_graph(
      c, precision,
      [&](cudaStream_t cs) {
        return sbe_rk4_step(c, P, C, D, Ek0, dEk, dt, precision, src_out, (void*)cs);
      },
      out, n_kernels);
}

int sbe_graph_launch(SbeGraph* g, void* stream) {
  if (!g || !g->exec) return fail(SBE_ERR_ARG, "sbe_graph_launch: null graph");
  return cuda_check(cudaGraphLaunch(g->exec, as_stream(stream)), "sbe_graph_launch");
}

int sbe_graph_destroy(SbeGraph* g) {
  if (!g) return SBE_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  delete g;
  return SBE_OK;
}

// ---- kernel timing ----------------------------------------------------------
int sbe_ctx_profile(SbeCtx* c, int enable) {
  if (!c) return fail(SBE_ERR_ARG, "sbe_ctx_profile: null");
  c->prof = enable ? 1 : 0;
  return SBE_OK;
}

int sbe_ctx_profile_read(SbeCtx* c, int category, double* total_ms, long long* launches) {
  if (!c || category < 0 || category > 3) return fail(SBE_ERR_ARG, "sbe_ctx_profile_read");
  double tot = 0.0;
  for (auto& pr : c->prof_ev[category]) {
    float ms = 0.f;
    cudaEventSynchronize(pr.second);
    cudaEventElapsedTime(&ms, pr.first, pr.second);
    tot += ms;
    c->ev_pool.push_back(pr.first);
    c->ev_pool.push_back(pr.second);
  }
  if (total_ms) *total_ms = tot;
  if (launches) *launches = (long long)c->prof_ev[category].size();
  c->prof_ev[category].clear();
  return SBE_OK;
}

// ---- charge balance ---------------------------------------------------------
int sbe_ctx_charge(SbeCtx* c, double* out, void* stream) {
  if (!c || !out) return fail(SBE_ERR_ARG, "sbe_ctx_charge: null argument");
  cudaStream_t s = as_stream(stream);
  int rc = cuda_check(cudaMemcpyAsync(out, c->charge, sizeof(double) * 2 * c->nw,
                                      cudaMemcpyDefault, s),
                      "sbe_ctx_charge: copy");
  if (rc) return rc;
  return cuda_check(cudaStreamSynchronize(s), "sbe_ctx_charge");
}

}  // extern "C"

namespace sbe {
// rates accumulation helper (MBPE/MBPH add to Win/Wout)
__global__ void k_add_rates(const double* wr, int nk, double* a, double* b, double* c, double* d) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  a[k] += wr[k];
  b[k] += wr[nk + k];
  c[k] += wr[2 * nk + k];
  d[k] += wr[3 * nk + k];
}

void add_rates(const double* wrate, int nk, double* a, double* b, double* cc, double* d,
               cudaStream_t s) {
  k_add_rates<<<(nk + 127) / 128, 128, 0, s>>>(wrate, nk, a, b, cc, d);
}
}  // namespace sbe
