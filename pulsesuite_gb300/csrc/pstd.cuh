// 1-D pseudo-spectral time-domain (PSTD) field grid and its coupling to the wires.
#pragma once
#include "sbe_ctx.cuh"

// The field grid: nx points (power of two), x_j = j dx - (nx - 1) dx / 2
// (GetSpaceArray, libpulsesuite/helpers.py:811-835), wavenumbers in FFT order
// (GetKArray, helpers.py:838-863).  Transverse fields E = (Ey, Ez), H = (Hz, Hy),
// longitudinal Ex.
struct SbePstd {
  int nx = 0, n1 = 0, n2 = 0, n_abc = 0;
  int dev = 0;
  double dx = 0, epsr = 1, abc_strength = 0;
  double2* tw = nullptr;    // nx: exp(-2 pi i j / nx)
  double* q = nullptr;      // nx: wavenumbers (FFT order)
  double* x = nullptr;      // nx: positions
  double* mask = nullptr;   // nx: absorbing-layer mask (1 in the interior)
  double2* work = nullptr;  // 2 nx: spectra of up to two fields
};

namespace sbe {
// Derivative passes.  in: nf (1 or 2) fields of nx c128; the epilogue of the
// last pass combines d = d/dx(in) (or the longitudinal field) with the outputs.
enum PstdEpi { PSTD_STORE = 0, PSTD_UPDATE = 1 };
struct PstdEpiArgs {
  int mode = PSTD_STORE;
  double2* out[2] = {nullptr, nullptr};
  const double2* jsrc[2] = {nullptr, nullptr};
  double a[2] = {1.0, 1.0};   // out += a * d
  double ja[2] = {0.0, 0.0};  // out += ja * J
  bool masked = false;
};
// kind 0: d/dx of nf fields; kind 1: longitudinal field of (rho, Px) -> one field.
int pstd_pipeline(SbePstd* p, int kind, const double2* in0, const double2* in1, int nf,
                  const PstdEpiArgs& epi, cudaStream_t s);
}  // namespace sbe
