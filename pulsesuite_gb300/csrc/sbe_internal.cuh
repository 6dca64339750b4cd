// Internal declarations shared by the CUDA translation units of libsbe_gb300.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/sbe_gb300.h"

namespace sbe {

// CODATA 2022 (the values scipy.constants carries, which the reference uses).
constexpr double kHbar = 1.0545718176461565e-34;
constexpr double kE0 = 1.602176634e-19;
constexpr double kEps0 = 8.8541878188e-12;
constexpr double kMe0 = 9.1093837139e-31;
constexpr double kKb = 1.380649e-23;
constexpr double kPi = 3.141592653589793;
constexpr double kTwoPi = 2.0 * 3.141592653589793;
constexpr double kEuler = 0.5772156649015329;
constexpr double kSmall = 1e-200;   // SBEs.py:4705
constexpr double kQwSmall = 1e-100; // qwoptics.py:598

// Per-wire data visible to kernels.  Offsets are in elements of the packed
// buffers (matrices: sum of Nk^2; vectors: sum of Nk; r-vectors: sum of Nr;
// De/Dh: sum of (2Nk+1)*Nk; Expikr: sum of Nk*Nr).
struct WireDev {
  int nk, nr, flags, w;      // w = 1-based wire index
  int yw, zsign;             // yw(w) and (-1)^w
  int dnk, pad;
  long long off_mat, off_vec, off_r, off_dd, off_kr, off_tab;  // off_tab: shared-table set
  double L, dkr, dr_grid, Delta0, gap, me, mh, HO;
  double gam_e, gam_h, gam_eh, epsr, Oph, Gph, temp, Edc;
  double dcv, alphae, alphah, ehint, area, qc;
  double vscale, n0ph, nmax;   // phonon Vscale, Bose N0, screening clamp
  double pol_scale;            // 2 ehint / (area L)
  double rho_scale;            // 2 e0 ehint / area
  // FP32 coupling constants of the mixed path (host-rounded once): the dipole
  // term -ehint Xcv of Heh as the x, y, z weights ed_x (odd k; even k: -ed_x),
  // ed_y, ed_z
  float ed_x, ed_y, ed_z, padf;
  // spontaneous emission (Recomb): photon-energy grid of InitializeEmission
  // (emis_nw midpoints, spacing emis_dhw) and its table at off_emis
  int emis_nw, pad3;
  double emis_dhw;
  long long off_emis;
};

struct SbeCtxImpl;

// Error helpers (thread-local message).
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// ----- complex helpers ----------------------------------------------------
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ inline double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ inline double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }

}  // namespace sbe
