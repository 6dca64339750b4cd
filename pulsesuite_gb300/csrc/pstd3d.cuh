// 3-D PSTD field grid (pstd3d.cu), shared with the 3-D wire coupling (couple.cu).
#pragma once
#include "sbe_ctx.cuh"

// Grid nx x ny x nz (C order, z fastest); per axis positions (GetSpaceArray,
// typespace.py:815-849), FFT-order wavenumbers (GetKArray, helpers.py:838-863), the
// absorbing mask and the twiddles of the axis FFT; one work array for the transforms.
struct SbePstd3 {
  int n[3] = {0, 0, 0};         // nx, ny, nz
  int n_abc[3] = {0, 0, 0};
  int fp32 = 0;
  double d[3] = {0, 0, 0};
  double epsr = 1.0, abc = 0.0;
  long long N = 0;
  void* arena = nullptr;
  double* x[3] = {nullptr, nullptr, nullptr};     // positions
  double* q[3] = {nullptr, nullptr, nullptr};     // wavenumbers (FFT order)
  double* mask[3] = {nullptr, nullptr, nullptr};  // absorbing mask per axis
  double2* tw[3] = {nullptr, nullptr, nullptr};   // exp(-2 pi i j / n), j < n
  float2* twf[3] = {nullptr, nullptr, nullptr};
  float2* qb[3] = {nullptr, nullptr, nullptr};    // q of bit-reversed positions, FP32 pairs
  void* work = nullptr;         // up to 10 fields of N complex (FP64) work
};

namespace sbe {
// Field half-steps of one leapfrog step (pstd3d.cu): the H update leaves the work
// array holding the forward transform of the new H when the transform planes fit in
// shared memory, and the E update that follows starts from it; nothing else may use
// the work array in between.
int pstd3_update_h_fwd(SbePstd3* p, const double2* E, double2* H, double dt, cudaStream_t s);
int pstd3_update_e_from_work(SbePstd3* p, double2* E, const double2* H, const double2* J,
                             double dt, cudaStream_t s);
}  // namespace sbe
