// Spontaneous emission (flag Recomb): InitializeEmission / SpontEmission of
// emission.py:35-131 with Ec (:133-171), SpontIntegral (:174-198) and rho0
// (:201-217); the decay ne <- ne exp(-Rsp nh dt), nh <- nh exp(-Rsp ne dt) of the
// relaxation (SBEs.py:5322-5325) is applied in k_relax_norm.
#include <cmath>
#include <vector>

#include "sbe_ctx.cuh"
#include "sbe_internal.cuh"

namespace sbe {

namespace {
constexpr double kC0 = 299792458.0;
// emission.py:28: the emission module keeps its own temperature (77 K); SBEs.py
// never sets it, so the tables use it whatever the wire's temperature is
constexpr double kEmissionTemp = 77.0;
}  // namespace

// InitializeEmission (emission.py:35-91) with CalcHOmega (:220-255): the
// photon-energy midpoints HOmega_n = (n + 1/2) d followed by the pre-calculated
// square array (2 nw values); dhw = HOmega_1 - HOmega_0 as SpontIntegral takes it.
std::vector<double> emission_table(const WireDev& W, int* nw, double* dhw) {
  const double dcv = std::fabs(W.dcv), ehint = W.ehint, geh = W.gam_eh;
  const double kBT = kKb * kEmissionTemp, hg = kHbar * geh;
  const double hwmax = (kBT + hg) * 4.0;
  const double d = std::min(kBT, hg) / 20.0;
  const int n = (int)std::ceil(hwmax / d);
  *nw = n;
  std::vector<double> how(std::max(n, 0)), sq(std::max(n, 0));
  for (int i = 0; i < n; ++i) how[i] = 0.0 + (i + 0.5) * d;
  for (int i = 0; i < n; ++i) {
    const double lrtz = (hg / kPi) / (how[i] * how[i] + hg * hg);   // usefulsubs.Lrtz
    sq[i] = 3.0 * dcv * dcv * ehint / kEps0 / std::sqrt(W.epsr) * ehint / kHbar * lrtz *
            std::exp(-how[i] / kKb / kEmissionTemp);
  }
  *dhw = n > 1 ? how[1] - how[0] : d;
  how.insert(how.end(), sq.begin(), sq.end());
  return how;
}

namespace {

// One block per (k, wire): Ec[k] (emission.py:133-171, with the reference's lower-
// triangular V: V[i][k] = v[i - k] for i >= k, V[k][k] = v[0]), Ek = gap + Ee + Eh +
// Ec, Rsp[k] = sum_n (H_n + Ek) rho0(H_n + Ek) square_n dhw.  ne, nh: real parts.
__global__ void __launch_bounds__(256) k_spont(const WireDev* wires, int w_only,
                                               const double2* nev, const double2* nhv,
                                               const double* vs, const double* Ee,
                                               const double* Eh, const double* emis,
                                               double* rsp) {
  const WireDev W = wires[w_only >= 0 ? w_only : blockIdx.y];
  const int n = W.nk, k = blockIdx.x;
  if (k >= n || !(W.flags & SBE_F_RECOMB)) return;
  const double* veh = vs + 3 * W.off_vec;
  const double* vee = veh + n;
  const double* vhh = veh + 2 * n;
  __shared__ double red[256];
  // Ec: sum_i ne_i (Vee[k][k] - Vee[i][k]) + nh_i (Vhh[k][k] - Vhh[i][k]) and
  // sum_i (ne_i Veh[k][k] idel[i][k] - nh_i Veh[k][k] idel[i][k])
  double s1 = 0.0, s2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double a = nev[W.off_vec + i].x, b = nhv[W.off_vec + i].x;
    const double vee_ik = i >= k ? vee[i - k] : 0.0, vhh_ik = i >= k ? vhh[i - k] : 0.0;
    s1 += a * (vee[0] - vee_ik) + b * (vhh[0] - vhh_ik);
    const double idel = i == k ? 0.0 : 1.0;
    s2 += a * veh[0] * idel - b * veh[0] * idel;
  }
  red[threadIdx.x] = s1;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double sum1 = red[0];
  __syncthreads();
  red[threadIdx.x] = s2;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double ec = (sum1 + red[0]) - veh[0];
  const double ek = W.gap + Ee[W.off_vec + k] + Eh[W.off_vec + k] + ec;
  __syncthreads();
  // SpontIntegral
  const double* how = emis + W.off_emis;
  const double* sq = how + W.emis_nw;
  const double rho = ((kC0 * kC0 * kC0) * (kPi * kPi)) * (kHbar * kHbar * kHbar);
  double acc = 0.0;
  for (int i = threadIdx.x; i < W.emis_nw; i += blockDim.x) {
    const double hw = how[i] + ek;
    acc += hw * (hw * hw / rho) * sq[i];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) rsp[W.off_vec + k] = red[0] * W.emis_dhw;
}

}  // namespace

void launch_spont(SbeCtx* c, int w_only, cudaStream_t s) {
  bool any = false;
  for (int w = 0; w < c->nw; ++w)
    if ((w_only < 0 || w == w_only) && (c->wires[w].flags & SBE_F_RECOMB)) any = true;
  if (!any) return;
  const int nk = w_only >= 0 ? c->wires[w_only].nk : c->nk_max;
  k_spont<<<dim3(nk, w_only >= 0 ? 1 : c->nw), 256, 0, s>>>(
      c->d_wires, w_only, c->ne, c->nh, c->vs, c->Ee, c->Eh, c->emis, c->rsp);
}

}  // namespace sbe
