// DC transport (flag DCTrans): dcfield.py:1154-1236 Transport of C3, D3 and p3
// after the relaxation (SBEs.py:5686-5690).  The reference shifts every matrix in
// momentum through ifft2(fft2(X) exp(-i (Y_a + Y_b) dk)) (LF on; with LF off only
// the diagonal through the 1-D transforms), dk = -e (Edc + Re Ex(q = 0)) dt / hbar and
// Y the centred array GetKArray(Nk, (Nk - 1) dky) (dcfield.py:39-58, 778) paired with
// the transforms' natural order as written.  The shift is the circulant
// S[a][b] = s((a - b) mod Nk), s(m) = (1/Nk) sum_n exp(-i Y_n dk) exp(2 pi i n m / Nk),
// so the 2-D shift is S X S^T: two complex FP64 GEMMs per matrix.
#include <cmath>

#include "sbe_ctx.cuh"
#include "sbe_internal.cuh"

namespace sbe {

bool any_dc(const SbeCtx* c) {
  for (const auto& W : c->wires)
    if (W.flags & SBE_F_DCTRANS) return true;
  return false;
}

namespace {

// s(m) of every wire with DCTrans: one block per (m, wire); Ek in q order (q = 0 at
// index 0 of the wire's x component)
__global__ void __launch_bounds__(256) k_dc_kernel(const WireDev* wires, const double2* Ek,
                                                   double dt, double2* dcs) {
  const WireDev W = wires[blockIdx.y];
  const int n = W.nk, m = blockIdx.x;
  if (m >= n || !(W.flags & SBE_F_DCTRANS)) return;
  const double eac = Ek[3 * W.off_r].x;
  const double dk = -kE0 * (W.Edc + eac) / kHbar * dt;
  // Y = GetKArray(Nk, (Nk - 1) dky): k_n = n dY, Y_n = k_n - k_{Nk/2}; dky = ky[2] - ky[1]
  const double dY = n > 1 ? kTwoPi / ((double)(n - 1) * W.dkr) : 1.0;   // L = 0: dk = 1
  const double yc = (double)(n / 2) * dY;
  double sr = 0.0, si = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double y = (double)j * dY - yc;
    double s1, c1, s2, c2;
    sincos(-y * dk, &s1, &c1);
    const long long jm = ((long long)j * m) % n;
    sincos(kTwoPi * (double)jm / (double)n, &s2, &c2);
    sr += c1 * c2 - s1 * s2;
    si += c1 * s2 + s1 * c2;
  }
  __shared__ double red[2][256];
  red[0][threadIdx.x] = sr;
  red[1][threadIdx.x] = si;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    dcs[W.off_vec + m] = make_double2(red[0][0] / n, red[1][0] / n);
}

// S of every wire: the circulant for DCTrans with LF, the identity otherwise (the
// GEMMs then leave the matrix unchanged exactly)
__global__ void k_dc_smat(const WireDev* wires, const double2* dcs, double2* S) {
  const WireDev W = wires[blockIdx.z];
  const int n = W.nk;
  const int b = blockIdx.x * blockDim.x + threadIdx.x, a = blockIdx.y;
  if (a >= n || b >= n) return;
  const bool shift = (W.flags & SBE_F_DCTRANS) && (W.flags & SBE_F_LF);
  double2 v = make_double2(a == b ? 1.0 : 0.0, 0.0);
  if (shift) v = dcs[W.off_vec + ((a - b) % n + n) % n];
  S[W.off_mat + (long long)a * n + b] = v;
}

// LF off: the diagonal alone, d'[a] = sum_c s(a - c) X[c][c] (into tmp)
__global__ void k_dc_diag(const WireDev* wires, const double2* dcs, const double2* X,
                          double2* tmp) {
  const WireDev W = wires[blockIdx.y];
  const int n = W.nk, a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n || !(W.flags & SBE_F_DCTRANS) || (W.flags & SBE_F_LF)) return;
  double2 acc = make_double2(0.0, 0.0);
  for (int cidx = 0; cidx < n; ++cidx)
    acc = cadd(acc, cmul(dcs[W.off_vec + ((a - cidx) % n + n) % n],
                         X[W.off_mat + (long long)cidx * n + cidx]));
  tmp[W.off_vec + a] = acc;
}

__global__ void k_dc_diag_store(const WireDev* wires, const double2* tmp, double2* X) {
  const WireDev W = wires[blockIdx.y];
  const int n = W.nk, a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n || !(W.flags & SBE_F_DCTRANS) || (W.flags & SBE_F_LF)) return;
  X[W.off_mat + (long long)a * n + a] = tmp[W.off_vec + a];
}

}  // namespace

void launch_dc_transport(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek,
                         double dt, cudaStream_t s) {
  if (!any_dc(c)) return;
  const int nk = c->nk_max;
  k_dc_kernel<<<dim3(nk, c->nw), 256, 0, s>>>(c->d_wires, Ek, dt, c->dcs);
  bool lf = false, nolf = false;
  for (const auto& W : c->wires)
    if (W.flags & SBE_F_DCTRANS) (W.flags & SBE_F_LF ? lf : nolf) = true;
  double2* X[3] = {C, D, P};
  if (lf) {
    // S into dA (the dephasing contraction matrices are not used after the RHS), the
    // product S X into dP (the RHS outputs are consumed by then), then X = (S X) S^T;
    // only the wires with DCTrans and LF take part (the others keep X untouched)
    double2* S = c->dA;
    double2* T = c->dP;
    k_dc_smat<<<dim3((nk + 127) / 128, nk, c->nw), 128, 0, s>>>(c->d_wires, c->dcs, S);
    for (int i = 0; i < 3; ++i) {
      GemmBatch b{};
      b.nterms = 1;
      b.t[0] = Term{S, X[i], OP_N, OP_N, 0, make_double2(1.0, 0.0)};
      b.out = T;
      b.flag_mask = SBE_F_DCTRANS | SBE_F_LF;
      launch_gemm64(c->d_wires, c->nw, nk, b, true, 0, s);
      GemmBatch b2{};
      b2.nterms = 1;
      b2.t[0] = Term{T, S, OP_N, OP_T, 0, make_double2(1.0, 0.0)};
      b2.out = X[i];
      b2.flag_mask = SBE_F_DCTRANS | SBE_F_LF;
      launch_gemm64(c->d_wires, c->nw, nk, b2, true, 0, s);
    }
  }
  if (nolf) {
    double2* tmp[3] = {c->ne, c->nh, reinterpret_cast<double2*>(c->wrate)};
    const dim3 g((nk + 127) / 128, c->nw);
    for (int i = 0; i < 3; ++i) {
      k_dc_diag<<<g, 128, 0, s>>>(c->d_wires, c->dcs, X[i], tmp[i]);
      k_dc_diag_store<<<g, 128, 0, s>>>(c->d_wires, tmp[i], X[i]);
    }
  }
}

}  // namespace sbe
