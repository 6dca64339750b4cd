// Time stepping of every wire: the reference leapfrog update, relaxation and
// charge normalisation, RK4 stage updates, the polarisation / charge sources and
// the field resampling between the propagation grid and the wire grid (FP64).
#include "sbe_ctx.cuh"

namespace sbe {

// ---------------------------------------------------------------------------
// SBEs.py:5673-5675: X3 = X1 + 2 dt dX for P, C, D; X3 is written into the
// level-1 buffers (their old contents are not needed any more).
__global__ void k_leap_update(const WireDev* wires, double2* L1p, const double2* L2p,
                              const double2* dP, double2* L1c, const double2* L2c,
                              const double2* dC, double2* L1d, const double2* L2d,
                              const double2* dD, double dt) {
  const WireDev W = wires[blockIdx.y];
  long long n = (long long)W.nk * W.nk;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long o = W.off_mat + i;
    double2 a = L2p[o], d = dP[o];
    L1p[o] = make_double2(a.x + d.x * dt * 2.0, a.y + d.y * dt * 2.0);
    a = L2c[o]; d = dC[o];
    L1c[o] = make_double2(a.x + d.x * dt * 2.0, a.y + d.y * dt * 2.0);
    a = L2d[o]; d = dD[o];
    L1d[o] = make_double2(a.x + d.x * dt * 2.0, a.y + d.y * dt * 2.0);
  }
}

// SBEs.py:5704-5706 and _checkin (5070-5080): with X3 held in level 1,
// new level1 = old level2, level2 = (old level2 + X3)/2, level3 = X3.
__global__ void k_leap_shuffle(const WireDev* wires, double2* L1, double2* L2, double2* L3) {
  const WireDev W = wires[blockIdx.y];
  long long n = (long long)W.nk * W.nk;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long o = W.off_mat + i;
    double2 a = L2[o], b = L1[o];
    L1[o] = a;
    L2[o] = make_double2((a.x + b.x) / 2.0, (a.y + b.y) / 2.0);
    L3[o] = b;
  }
}

// phonons.py:140-268 MBPE / MBPH for row k of every wire, with the screened
// VC and E1D of the preparation: Vep = VC[:,:,1]/E1D*Vscale (VC already
// divided by E1D once: the quirk is kept).  ne, nh are Re(diag) of C3, D3.
__global__ void k_phonon_rates(const WireDev* wires, int w_only, const double2* nev,
                               const double2* nhv, const double* vs, const double* eps,
                               const double* EP, const double* HP, double* wrate) {
  const WireDev W = wires[w_only >= 0 ? w_only : blockIdx.y];
  const int nk = W.nk;
  int k = blockIdx.x;
  if (k >= nk) return;
  if (!(W.flags & SBE_F_PHONON)) {
    // no phonon rates: the carrier-carrier rates (EHs) are added to zeros
    if (threadIdx.x < 4) wrate[4 * W.off_vec + threadIdx.x * nk + k] = 0.0;
    return;
  }
  const double* v1 = vs + 3 * W.off_vec + nk;
  const double* v2 = vs + 3 * W.off_vec + 2 * nk;
  const double* ep = eps + W.off_vec;
  const double* EPw = EP + W.off_mat;
  const double* HPw = HP + W.off_mat;
  double wie = 0.0, woe = 0.0, wih = 0.0, woh = 0.0;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    double ne_i = nev[W.off_vec + i].x;
    double nh_i = nhv[W.off_vec + i].x;
    // electrons: Vep[k, i] (nonzero for k >= i)
    int d = k - i;
    double vep = (d >= 0 ? v1[d] : 0.0) / ep[d >= 0 ? d : -d] * W.vscale;
    wie += vep * ne_i * EPw[(long long)k * nk + i];
    woe += vep * (1.0 - ne_i) * EPw[(long long)i * nk + k];
    // holes: Vhp[i, k] (nonzero for i >= k)
    int e = i - k;
    double vhp = (e >= 0 ? v2[e] : 0.0) / ep[e >= 0 ? e : -e] * W.vscale;
    wih += vhp * nh_i * HPw[(long long)k * nk + i];
    woh += vhp * (1.0 - nh_i) * HPw[(long long)i * nk + k];
  }
  __shared__ double red[4][128];
  red[0][threadIdx.x] = wie;
  red[1][threadIdx.x] = woe;
  red[2][threadIdx.x] = wih;
  red[3][threadIdx.x] = woh;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int j = 0; j < 4; ++j) red[j][threadIdx.x] += red[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 4) wrate[4 * W.off_vec + threadIdx.x * nk + k] = red[threadIdx.x][0];
}

// SBEs.py:5677-5702 + 5276-5325: relaxation of the diagonals with the phonon
// in/out rates, then the charge normalisation ne = |C_kk| scaled to the common
// mean.  One block per wire.  The normalised occupations are left in ne/nh for
// the sources.
__device__ __forceinline__ double2 cexp_d(double2 z) {
  const double m = exp(z.x);
  double sn, cs;
  sincos(z.y, &sn, &cs);
  return make_double2(m * cs, m * sn);
}

// mode 0: relaxation and normalisation; 1: relaxation only (the relaxed complex
// diagonals back into C3, D3); 2: normalisation only.
__global__ void k_relax_norm(const WireDev* wires, double2* C3, double2* D3, const double* wrate,
                             const double* rsp, double dt, double2* ne_out, double2* nh_out,
                             double* charge, int mode) {
  const WireDev W = wires[blockIdx.x];
  const int nk = W.nk;
  const bool relax = mode != 2 && (W.flags & (SBE_F_PHONON | SBE_F_EHS)) != 0;
  // the decay is part of the relaxation, which runs only with Phonon or EHs
  // (SBEs.py:5677, 5322)
  const bool recomb = relax && (W.flags & SBE_F_RECOMB) != 0;
  __shared__ double red[2][256];
  double se = 0.0, sh = 0.0;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    long long o = W.off_mat + (long long)k * nk + k;
    double2 ne = C3[o], nh = D3[o];
    if (relax) {
      const double* wr = wrate + 4 * W.off_vec;
      double wie = wr[k], woe = wr[nk + k], wih = wr[2 * nk + k], woh = wr[3 * nk + k];
      double We = wie + woe, Wh = wih + woh;
      double ee = exp(-We * dt), ep = exp(We * dt);
      double he = exp(-Wh * dt), hp = exp(Wh * dt);
      double den_e = We + kSmall, den_h = Wh + kSmall;
      ne = make_double2(ee * ((-1 + ep + ne.x) * wie + ne.x * woe) / den_e,
                        ee * (ne.y * wie + ne.y * woe) / den_e);
      nh = make_double2(he * ((-1 + hp + nh.x) * wih + nh.x * woh) / den_h,
                        he * (nh.y * wih + nh.y * woh) / den_h);
    }
    if (recomb) {
      // SBEs.py:5322-5325: ne exp(-Rsp nh dt), then nh exp(-Rsp ne dt) with the new ne
      // (complex occupations, complex exponential)
      const double r = rsp[W.off_vec + k];
      ne = cmul(ne, cexp_d(make_double2(-r * nh.x * dt, -r * nh.y * dt)));
      nh = cmul(nh, cexp_d(make_double2(-r * ne.x * dt, -r * ne.y * dt)));
    }
    if (mode == 1) {
      C3[o] = ne;
      D3[o] = nh;
      continue;
    }
    double ae = hypot(ne.x, ne.y), ah = hypot(nh.x, nh.y);
    ne_out[W.off_vec + k] = make_double2(ae, 0.0);
    nh_out[W.off_vec + k] = make_double2(ah, 0.0);
    se += ae;
    sh += ah;
  }
  if (mode == 1) return;   // block-uniform
  red[0][threadIdx.x] = se;
  red[1][threadIdx.x] = sh;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  double sum_e = red[0][0], sum_h = red[1][0];
  if (threadIdx.x == 0) {
    // the carrier numbers before the normalisation: their difference is what this
    // step's relaxation and rounding left of the electron-hole balance
    charge[2 * blockIdx.x] = sum_e;
    charge[2 * blockIdx.x + 1] = sum_h;
  }
  double total = (sum_e + sum_h) / 2.0;
  double fe = total / (sum_e + kSmall), fh = total / (sum_h + kSmall);
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    long long o = W.off_mat + (long long)k * nk + k;
    double ae = ne_out[W.off_vec + k].x * fe, ah = nh_out[W.off_vec + k].x * fh;
    ne_out[W.off_vec + k] = make_double2(ae, 0.0);
    nh_out[W.off_vec + k] = make_double2(ah, 0.0);
    C3[o] = make_double2(ae, 0.0);
    D3[o] = make_double2(ah, 0.0);
  }
}

void launch_relax_norm(SbeCtx* c, double2* P3, double2* C3, double2* D3, const double2* Ek,
                       double dt, cudaStream_t s) {
  launch_extract_diag(c, C3, D3, s);
  k_phonon_rates<<<dim3(c->nk_max, c->nw), 128, 0, s>>>(c->d_wires, -1, c->ne, c->nh, c->vs,
                                                        c->eps, c->EP, c->HP, c->wrate);
  launch_mbc_rates(c, -1, s);
  launch_relax_only(c, P3, C3, D3, Ek, dt, s);
}

// relaxation (rates already in c->wrate), DC transport and normalisation
// (SBEs.py:5677-5702: relaxation, Transport of C3, D3, p3, charge normalisation)
void launch_relax_only(SbeCtx* c, double2* P3, double2* C3, double2* D3, const double2* Ek,
                       double dt, cudaStream_t s) {
  if (!any_dc(c)) {
    k_relax_norm<<<c->nw, 256, 0, s>>>(c->d_wires, C3, D3, c->wrate, c->rsp, dt, c->ne, c->nh,
                                       c->charge, 0);
    return;
  }
  k_relax_norm<<<c->nw, 256, 0, s>>>(c->d_wires, C3, D3, c->wrate, c->rsp, dt, c->ne, c->nh,
                                     c->charge, 1);
  launch_dc_transport(c, P3, C3, D3, Ek, dt, s);
  k_relax_norm<<<c->nw, 256, 0, s>>>(c->d_wires, C3, D3, c->wrate, c->rsp, dt, c->ne, c->nh,
                                     c->charge, 2);
}

void launch_phonon_rates_one(SbeCtx* c, int w, cudaStream_t s) {
  k_phonon_rates<<<dim3(c->wires[w].nk, 1), 128, 0, s>>>(c->d_wires, w, c->ne, c->nh, c->vs,
                                                         c->eps, c->EP, c->HP, c->wrate);
}

void launch_leapfrog(SbeCtx* c, double2* const* st, const double2* Ek, double dt,
                     cudaStream_t s) {
  // st: YY1, YY2, YY3, CC1, CC2, CC3, DD1, DD2, DD3
  int blocks = (int)std::min<long long>(((long long)c->nk_max * c->nk_max + 255) / 256, 4096);
  dim3 g(blocks, c->nw);
  k_leap_update<<<g, 256, 0, s>>>(c->d_wires, st[0], st[1], c->dP, st[3], st[4], c->dC, st[6],
                                  st[7], c->dD, dt);
  launch_relax_norm(c, st[0], st[3], st[6], Ek, dt, s);
}

void launch_leap_shuffle(SbeCtx* c, double2* const* st, cudaStream_t s) {
  int blocks = (int)std::min<long long>(((long long)c->nk_max * c->nk_max + 255) / 256, 4096);
  dim3 g(blocks, c->nw);
  k_leap_shuffle<<<g, 256, 0, s>>>(c->d_wires, st[0], st[1], st[2]);
  k_leap_shuffle<<<g, 256, 0, s>>>(c->d_wires, st[3], st[4], st[5]);
  k_leap_shuffle<<<g, 256, 0, s>>>(c->d_wires, st[6], st[7], st[8]);
}

// ---------------------------------------------------------------------------
// Sources.  qwoptics.py:50-76 (QWPolarization3) with Xvc0[kh,ke] = dcv (-1)^kh,
// Yvc0 = dcv, Zvc0 = -dcv (qwoptics.py:618-626) reduces to G = p E (E = Expikr)
// and column sums over kh; qwoptics.py:361-374 (QWRho5) to C E and conj(D) E.
// Output per wire: 5 x Nr c128 [Px, Py, Pz, re, rh] in real space (the
// reference's FFTG here is undone by the iFFTG of QW2Prop).
__global__ void k_src_reduce(const WireDev* wires, int w_only, const double2* expikr,
                             const double2* G, long long tot_kr, const double* win, double2* src) {
  const WireDev W = wires[w_only >= 0 ? w_only : blockIdx.y];
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= W.nr) return;
  const int nk = W.nk, nr = W.nr;
  const double2* E = expikr + W.off_kr;
  const double2* Gp = G + W.off_kr;
  const double2* Gc = G + tot_kr + W.off_kr;
  const double2* Gd = G + 2 * tot_kr + W.off_kr;
  double sx = 0.0, sy = 0.0;
  double2 se = make_double2(0, 0), sh = make_double2(0, 0);
  for (int k = 0; k < nk; ++k) {
    double2 e = cconj(E[(long long)k * nr + r]);
    double2 gp = Gp[(long long)k * nr + r];
    double re_part = e.x * gp.x - e.y * gp.y;
    sx += (k & 1) ? -re_part : re_part;
    sy += re_part;
    se = cadd(se, cmul(e, Gc[(long long)k * nr + r]));
    sh = cadd(sh, cmul(e, Gd[(long long)k * nr + r]));
  }
  double w = win[W.off_r + r];
  double2* out = src + 5 * W.off_r;
  bool optics = (W.flags & SBE_F_OPTICS) != 0;
  double px = optics ? (W.dcv * sx) * w : 0.0;
  double py = optics ? (W.dcv * sy) * w * W.yw : 0.0;
  double pz = optics ? (-W.dcv * sy) * w * W.zsign : 0.0;
  out[r] = make_double2(px * 2 * W.ehint / W.area / W.L, 0.0);
  out[nr + r] = make_double2(py * 2 * W.ehint / W.area / W.L, 0.0);
  out[2 * nr + r] = make_double2(pz * 2 * W.ehint / W.area / W.L, 0.0);
  out[3 * nr + r] = cscale(se, w / (2.0 * W.L));
  out[4 * nr + r] = cscale(sh, w / (2.0 * W.L));
}

// qwoptics.py:1062-1068 boundary-mean subtraction and renormalisation, then
// SBEs.py:5749-5750 (x 2 e0 ehint / area).  One block per wire.
__global__ void k_src_final(const WireDev* wires, int w_only, const double* r, const double2* ne,
                            const double2* nh, double2* src) {
  const WireDev W = wires[w_only >= 0 ? w_only : blockIdx.x];
  const int nr = W.nr, nk = W.nk;
  double2* re = src + 5 * W.off_r + 3 * nr;
  double2* rh = re + nr;
  const bool lf = (W.flags & SBE_F_LF) != 0;
  if (!lf) {
    for (int j = threadIdx.x; j < nr; j += blockDim.x) {
      re[j] = make_double2(0, 0);
      rh[j] = make_double2(0, 0);
    }
    return;
  }
  __shared__ double red[4][256];
  double a = 0, b = 0, c = 0, d = 0;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    a += hypot(ne[W.off_vec + k].x, ne[W.off_vec + k].y);
    b += hypot(nh[W.off_vec + k].x, nh[W.off_vec + k].y);
  }
  // sum(re[0:10]) + sum(re[Nr-10:Nr]): an index in both slices counts twice
  for (int j = threadIdx.x; j < nr; j += blockDim.x) {
    int m = (j < 10 ? 1 : 0) + (j >= nr - 10 ? 1 : 0);
    c += m * re[j].x;
    d += m * rh[j].x;
  }
  red[0][threadIdx.x] = a; red[1][threadIdx.x] = b; red[2][threadIdx.x] = c; red[3][threadIdx.x] = d;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    __syncthreads();
  }
  double NeT = red[0][0] + 1e-50, NhT = red[1][0] + 1e-50;
  double be = red[2][0] / 20.0, bh = red[3][0] / 20.0;
  __syncthreads();
  double ae = 0, ah = 0;
  for (int j = threadIdx.x; j < nr; j += blockDim.x) {
    double2 x = re[j], y = rh[j];
    x.x -= be;
    y.x -= bh;
    re[j] = x;
    rh[j] = y;
    ae += hypot(x.x, x.y);
    ah += hypot(y.x, y.y);
  }
  red[0][threadIdx.x] = ae;
  red[1][threadIdx.x] = ah;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  const double* rw = r + W.off_r;
  double dr = rw[1] - rw[0];
  double fe = NeT / (red[0][0] * dr + kQwSmall), fh = NhT / (red[1][0] * dr + kQwSmall);
  for (int j = threadIdx.x; j < nr; j += blockDim.x) {
    double2 x = cscale(re[j], fe), y = cscale(rh[j], fh);
    re[j] = make_double2(2.0 * kE0 * x.x / W.area * W.ehint, 2.0 * kE0 * x.y / W.area * W.ehint);
    rh[j] = make_double2(2.0 * kE0 * y.x / W.area * W.ehint, 2.0 * kE0 * y.y / W.area * W.ehint);
  }
}

void launch_sources(SbeCtx* c, const double2* P, const double2* C, const double2* D,
                    const double2* ne, const double2* nh, double2* src, cudaStream_t s,
                    int w_only) {
  const double2 one = make_double2(1.0, 0.0);
  const double2* mats[3] = {P, C, D};
  for (int i = 0; i < 3; ++i) {
    GemmBatch b{};
    b.w_only = w_only;
    b.nterms = 1;
    b.t[0].A = mats[i];
    b.t[0].B = nullptr;
    b.t[0].opA = (i == 2) ? OP_C : OP_N;
    b.t[0].opB = OP_N;
    b.t[0].realA = 0;
    b.t[0].alpha = one;
    b.out = c->G + i * c->tot_kr;
    b.epi = 0;
    launch_sources_gemm64(c, b, s);
  }
  int nb = w_only >= 0 ? 1 : c->nw;
  (void)nb;
  k_src_reduce<<<dim3((c->nr_max + 127) / 128, nb), 128, 0, s>>>(c->d_wires, w_only, c->expikr,
                                                                c->G, c->tot_kr, c->window, src);
  k_src_final<<<nb, 256, 0, s>>>(c->d_wires, w_only, c->r, ne, nh, src);
}

// ---------------------------------------------------------------------------
// RK4 (classical tableau) over the packed state, FP64.  stage s in 1..4 uses the
// RHS in c->dP/dC/dD:  s=1: acc = k;   xs = X + dt/2 k
//                      s=2: acc += 2k; xs = X + dt/2 k
//                      s=3: acc += 2k; xs = X + dt k
//                      s=4: X += dt/6 (acc + k)
__global__ void k_rk4_axpy(long long n, int stage, double dt, double2* X, double2* acc,
                           double2* xs, const double2* k) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double2 kv = k[i];
    if (stage == 1) {
      acc[i] = kv;
      double2 x = X[i];
      xs[i] = make_double2(x.x + 0.5 * dt * kv.x, x.y + 0.5 * dt * kv.y);
    } else if (stage == 2 || stage == 3) {
      double2 a = acc[i];
      acc[i] = make_double2(a.x + 2.0 * kv.x, a.y + 2.0 * kv.y);
      double f = stage == 2 ? 0.5 * dt : dt;
      double2 x = X[i];
      xs[i] = make_double2(x.x + f * kv.x, x.y + f * kv.y);
    } else {
      double2 a = acc[i], x = X[i];
      X[i] = make_double2(x.x + dt / 6.0 * (a.x + kv.x), x.y + dt / 6.0 * (a.y + kv.y));
    }
  }
}

void launch_rk4_axpy(SbeCtx* c, int stage, double dt, double2* P, double2* C, double2* D,
                     cudaStream_t s) {
  long long n = c->tot_mat;
  int blocks = (int)std::min<long long>((n + 255) / 256, 8192);
  double2* X[3] = {P, C, D};
  double2* K[3] = {c->dP, c->dC, c->dD};
  for (int i = 0; i < 3; ++i)
    k_rk4_axpy<<<blocks, 256, 0, s>>>(n, stage, dt, X[i], c->kacc + i * n, c->xs + i * n, K[i]);
}

__global__ void k_stage_field(long long n, const double2* Ek0, const double2* dEk, double frac,
                              double2* out) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 a = Ek0[i];
  if (dEk) {
    double2 b = dEk[i];
    a.x += frac * b.x;
    a.y += frac * b.y;
  }
  out[i] = a;
}

void launch_stage_field(SbeCtx* c, const double2* Ek0, const double2* dEk, double frac,
                        cudaStream_t s) {
  long long n = 3 * c->tot_r;
  k_stage_field<<<(int)((n + 255) / 256), 256, 0, s>>>(n, Ek0, dEk, frac, c->ekst);
}

// ---------------------------------------------------------------------------
// Cubic spline resampling, spliner.py:153-189 rescale_1D_dpc with the
// Forsythe-Malcolm-Moler coefficients of spline_dpc (spliner.py:1329-1394) and
// the binary search of locate (spliner.py:1137-1167).  The coefficient solve
// is a sequential tridiagonal sweep: one thread per field.
__device__ void fmm_spline(int n, const double* x, const double2* y, double2* b, double2* c,
                           double2* d) {
  if (n < 3) {
    double2 s = cscale(csub(y[1], y[0]), 1.0 / (x[1] - x[0]));
    b[0] = s; b[1] = s;
    c[0] = c[1] = d[0] = d[1] = make_double2(0, 0);
    return;
  }
  d[0] = make_double2(x[1] - x[0], 0);
  c[1] = cscale(csub(y[1], y[0]), 1.0 / d[0].x);
  for (int i = 1; i < n - 1; ++i) {
    d[i] = make_double2(x[i + 1] - x[i], 0);
    b[i] = make_double2(2.0 * (d[i - 1].x + d[i].x), 0);
    double2 t = csub(y[i + 1], y[i]);
    c[i + 1] = make_double2(t.x / d[i].x, t.y / d[i].x);
    c[i] = csub(c[i + 1], c[i]);
  }
  b[0] = make_double2(-d[0].x, 0);
  b[n - 1] = make_double2(-d[n - 2].x, 0);
  c[0] = make_double2(0, 0);
  c[n - 1] = make_double2(0, 0);
  if (n != 3) {
    double2 c0 = csub(cscale(c[2], 1.0 / (x[3] - x[1])), cscale(c[1], 1.0 / (x[2] - x[0])));
    double2 cn = csub(cscale(c[n - 2], 1.0 / (x[n - 1] - x[n - 3])),
                      cscale(c[n - 3], 1.0 / (x[n - 2] - x[n - 4])));
    c[0] = cscale(c0, d[0].x * d[0].x / (x[3] - x[0]));
    c[n - 1] = cscale(cn, -d[n - 2].x * d[n - 2].x / (x[n - 1] - x[n - 4]));
  }
  for (int i = 1; i < n; ++i) {
    double t = d[i - 1].x / b[i - 1].x;
    b[i].x = b[i].x - t * d[i - 1].x;
    c[i] = csub(c[i], cscale(c[i - 1], t));
  }
  c[n - 1] = cscale(c[n - 1], 1.0 / b[n - 1].x);
  for (int i = n - 2; i >= 0; --i) {
    double2 t = csub(c[i], cscale(c[i + 1], d[i].x));
    c[i] = make_double2(t.x / b[i].x, t.y / b[i].x);
  }
  {
    double2 t = csub(y[n - 1], y[n - 2]);
    double2 u = cadd(c[n - 2], cscale(c[n - 1], 2.0));
    b[n - 1] = cadd(make_double2(t.x / d[n - 2].x, t.y / d[n - 2].x), cscale(u, d[n - 2].x));
  }
  for (int i = 0; i < n - 1; ++i) {
    double di = d[i].x;
    double2 t = csub(y[i + 1], y[i]);
    double2 u = cadd(c[i + 1], cscale(c[i], 2.0));
    b[i] = csub(make_double2(t.x / di, t.y / di), cscale(u, di));
    double2 v = csub(c[i + 1], c[i]);
    d[i] = make_double2(v.x / di, v.y / di);
    c[i] = cscale(c[i], 3.0);
  }
  c[n - 1] = cscale(c[n - 1], 3.0);
  d[n - 1] = d[n - 2];
}

__device__ int locate_dev(const double* xx, int n, double x) {
  if (x < xx[0]) return 0;
  if (x >= xx[n - 1]) return n - 1;
  int jl = 0, ju = n;
  while (ju - jl > 1) {
    int jm = (ju + jl) / 2;
    if (x >= xx[jm]) jl = jm;
    else ju = jm;
  }
  return jl;
}

__global__ void k_spline_coef(int n, const double* x, const double2* y, int nf, double2* coef) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double2* b = coef + (long long)f * 3 * n;
  fmm_spline(n, x, y + (long long)f * n, b, b + n, b + 2 * n);
}

// evaluate nf splines (knots x0, n0) at x1 (n1 points); values outside
// [min x0, max x0] are 0; optional window multiply and real part.
__global__ void k_spline_eval(int n0, const double* x0, const double2* y0, const double2* coef,
                              int n1, const double* x1, int nf, const double* win, int real_part,
                              double2* out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int f = blockIdx.y;
  if (j >= n1 || f >= nf) return;
  double lo = x0[0], hi = x0[0];
  for (int i = 1; i < n0; ++i) { lo = fmin(lo, x0[i]); hi = fmax(hi, x0[i]); }
  double u = x1[j];
  double2 v = make_double2(0, 0);
  if (u >= lo && u <= hi) {
    const double2* y = y0 + (long long)f * n0;
    const double2* b = coef + (long long)f * 3 * n0;
    const double2* c = b + n0;
    const double2* d = b + 2 * n0;
    int i = locate_dev(x0, n0, u);
    double dx = u - x0[i];
    double2 t = cadd(c[i], cscale(d[i], dx));
    t = cadd(b[i], cscale(t, dx));
    v = cadd(y[i], cscale(t, dx));
  }
  if (win) v = cscale(v, win[j]);
  if (real_part) v.y = 0.0;
  out[(long long)f * n1 + j] = v;
}

// FFTG (usefulsubs.py:2245-2268): F[q] = -(1/N) sum_j f[j] e^{-2 pi i q j / N}.
__global__ void k_fftg(int n, int nf, const double2* in, double2* out) {
  int q = blockIdx.x;
  int f = blockIdx.y;
  const double2* x = in + (long long)f * n;
  double sr = 0, si = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    long long qj = ((long long)q * j) % n;
    double s, c;
    sincospi(-2.0 * (double)qj / (double)n, &s, &c);
    double2 v = x[j];
    sr += v.x * c - v.y * s;
    si += v.x * s + v.y * c;
  }
  __shared__ double rr[128], ri[128];
  rr[threadIdx.x] = sr;
  ri[threadIdx.x] = si;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      rr[threadIdx.x] += rr[threadIdx.x + o];
      ri[threadIdx.x] += ri[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[(long long)f * n + q] = make_double2(-rr[0] / n, -ri[0] / n);
}

// Prop2QW on the context's scratch: the wire-grid part lives in the context's arena;
// the spline coefficients of the caller's grid (12 per point) in a context buffer that
// is allocated on the first call and grown only when a larger grid comes (cudaFree and
// cudaMalloc then wait for the device's pending work); calls of one context are
// ordered on its stream, so they share the scratch.
int launch_prop2qw(SbeCtx* c, int w, const double* RR, int n_rr, const double2* fin,
                   double2* out, cudaStream_t s) {
  const long long need = 12LL * n_rr;
  if (need > c->p2q_cap) {
    if (c->p2q_coef && cudaFree(c->p2q_coef) != cudaSuccess)
      return cuda_check(cudaGetLastError(), "prop2qw: release the smaller scratch");
    c->p2q_coef = nullptr;
    c->p2q_cap = 0;
    if (cudaMalloc(&c->p2q_coef, sizeof(double2) * need) != cudaSuccess)
      return fail(SBE_ERR_OOM, "prop2qw scratch");
    c->p2q_cap = need;
  }
  return launch_prop2qw_scratch(c, w, RR, n_rr, fin, out, c->p2q_coef, c->qscr, s);
}

// The same three launches as launch_prop2qw on scratch the caller provides:
// coef holds 12 n_rr and tmp 4 Nr complex values.  Allocates nothing.
int launch_prop2qw_scratch(SbeCtx* c, int w, const double* RR, int n_rr, const double2* fin,
                           double2* out, double2* coef, double2* tmp, cudaStream_t s) {
  const WireDev& W = c->wires[w];
  k_spline_coef<<<1, 32, 0, s>>>(n_rr, RR, fin, 4, coef);
  k_spline_eval<<<dim3((W.nr + 127) / 128, 4), 128, 0, s>>>(n_rr, RR, fin, coef, W.nr,
                                                           c->r + W.off_r, 4,
                                                           c->window + W.off_r, 1, tmp);
  k_fftg<<<dim3(W.nr, 4), 128, 0, s>>>(W.nr, 4, tmp, out);
  return cuda_check(cudaGetLastError(), "prop2qw (caller scratch)");
}

// qwoptics.py:760-805 charge renormalisation (Plasmonics).  mode 0: on the wire
// grid (re, rh -> |.| scaled to total); mode 1: on the propagation grid.
__global__ void k_plasmonics(int n, const double* grid, double2* a, double2* b, double* total_io,
                             int mode) {
  const double dx = grid[1] - grid[0];
  __shared__ double red[2][256];
  double sa = 0, sb = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double x = hypot(a[j].x, a[j].y), y = hypot(b[j].x, b[j].y);
    a[j] = make_double2(x, 0);
    b[j] = make_double2(y, 0);
    sa += x;
    sb += y;
  }
  red[0][threadIdx.x] = sa;
  red[1][threadIdx.x] = sb;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  double A = red[0][0], B = red[1][0];
  double total;
  if (mode == 0) {
    total = (A * dx + B * dx + kQwSmall) / 2.0;
    if (threadIdx.x == 0) *total_io = total;
  } else {
    total = *total_io;
  }
  double fa = total / (A * dx + kQwSmall), fb = total / (B * dx + kQwSmall);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    a[j] = make_double2(a[j].x * fa, 0);
    b[j] = make_double2(b[j].x * fb, 0);
  }
}

int launch_qw2prop(SbeCtx* c, int w, const double* RR, int n_rr, const double2* src,
                   double2* out, int plasmonics, cudaStream_t s) {
  // scratch in the context's arena (15 + 5 wire-grid columns and the total)
  const WireDev& W = c->wires[w];
  double2* coef = c->qscr;
  double2* tmp = coef + 15 * (size_t)c->nr_max;
  double* total = reinterpret_cast<double*>(tmp + 5 * (size_t)c->nr_max);
  cudaMemcpyAsync(tmp, src, sizeof(double2) * 5 * (size_t)W.nr, cudaMemcpyDeviceToDevice, s);
  const double* rw = c->r + W.off_r;
  if (plasmonics)
    k_plasmonics<<<1, 256, 0, s>>>(W.nr, rw, tmp + 3 * W.nr, tmp + 4 * W.nr, total, 0);
  k_spline_coef<<<1, 32, 0, s>>>(W.nr, rw, tmp, 5, coef);
  k_spline_eval<<<dim3((n_rr + 127) / 128, 5), 128, 0, s>>>(W.nr, rw, tmp, coef, n_rr, RR, 5,
                                                           nullptr, 0, out);
  if (plasmonics)
    k_plasmonics<<<1, 256, 0, s>>>(n_rr, RR, out + 3 * (size_t)n_rr, out + 4 * (size_t)n_rr,
                                   total, 1);
  return cuda_check(cudaGetLastError(), "qw2prop");
}

}  // namespace sbe

namespace sbe {
void launch_sources_final(SbeCtx* c, const double2* ne, const double2* nh, double2* src,
                          cudaStream_t s) {
  k_src_final<<<c->nw, 256, 0, s>>>(c->d_wires, -1, c->r, ne, nh, src);
}

void launch_sources_reduce(SbeCtx* c, const double2* ne, const double2* nh, double2* src,
                           cudaStream_t s) {
  k_src_reduce<<<dim3((c->nr_max + 127) / 128, c->nw), 128, 0, s>>>(c->d_wires, -1, c->expikr,
                                                                   c->G, c->tot_kr, c->window, src);
  k_src_final<<<c->nw, 256, 0, s>>>(c->d_wires, -1, c->r, ne, nh, src);
}
}  // namespace sbe
