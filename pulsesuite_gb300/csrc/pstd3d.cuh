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
  void* work = nullptr;         // up to 10 fields of N complex (FP64) work
};

