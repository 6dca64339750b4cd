// sbe_prop2qw_noalloc: Prop2QW (qwoptics.py:667-715) with its scratch in static
// device memory instead of stream-ordered allocations.
//
// Which callers need it: a host code that has handed all device memory to its own
// pool and must not allocate behind it (its allocations would fail or fragment the
// pool), and real-time loops that must not call cudaMallocAsync / cudaFreeAsync
// because those calls take the driver's allocator lock and may synchronise with
// other streams of the process.  sbe_prop2qw keeps 12 n_rr complex values of
// spline scratch in its context, allocated (cudaMalloc) on its first call and again
// whenever a larger grid comes; this variant uses one fixed array instead.
//
// Limits: n_rr <= SBE_NOALLOC_MAX_GRID (8192 propagation-grid points) and
// Nr <= SBE_NOALLOC_MAX_NR (2050 wire points, Nk <= 1024).  Larger calls are
// rejected with SBE_ERR_ARG / SBE_ERR_UNSUPPORTED before anything is launched.
//
// The scratch is one array per CUDA context: every context that loads this library
// on a device holds its own copy of the module and so of the array, until the
// context is destroyed or the process exits.  All calls made in one context share
// that array: two calls whose kernels overlap in time (different streams or host
// threads of the same context) race on it and give wrong results.  Calls on one
// stream are ordered and safe.  No element of the scratch needs to start at zero:
// every element a kernel reads was written earlier in the same call.
//
// Every call looks up the array's device address in the calling thread's current
// context with cudaGetSymbolAddress, so nothing is cached that a destroyed or reset
// context could leave stale.  The first call in a context may load the library's
// device code into it; make that first call before any stream capture.

#include "sbe_ctx.cuh"

namespace {

constexpr int kMaxGrid = SBE_NOALLOC_MAX_GRID;  // propagation-grid points (n_rr)
constexpr int kMaxNr = SBE_NOALLOC_MAX_NR;      // wire points (Nr = 2 Nk + 2, Nk <= 1024)
constexpr long long kCoefElems = 12LL * kMaxGrid;  // 4 fields x 3 spline coefficients
constexpr long long kTmpElems = 4LL * kMaxNr;      // 4 resampled fields on the wire grid

// 1.70 MB of complex128 scratch: spline coefficients, then the windowed fields.
static __device__ __align__(256) double2 g_prop2qw_scratch[kCoefElems + kTmpElems];

// Device address of the scratch in the current context (looked up on every call).
int scratch_ptr(double2** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_prop2qw_scratch);
  if (e != cudaSuccess || !p)
    return sbe::cuda_check(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                           "sbe_prop2qw_noalloc: cudaGetSymbolAddress");
  *out = static_cast<double2*>(p);
  return SBE_OK;
}

}  // namespace

extern "C" int sbe_prop2qw_noalloc(SbeCtx* c, int w, const double* RR, int n_rr,
                                   const double* fields_in, double* out, void* stream) {
  using namespace sbe;
  if (!c || w < 0 || w >= c->nw) return fail(SBE_ERR_ARG, "sbe_prop2qw_noalloc: bad context/wire");
  if (!RR || n_rr < 2 || !fields_in || !out)
    return fail(SBE_ERR_ARG, "sbe_prop2qw_noalloc: bad arguments");
  if (n_rr > kMaxGrid)
    return fail(SBE_ERR_ARG, "sbe_prop2qw_noalloc: n_rr = " + std::to_string(n_rr) +
                                 " exceeds the static scratch limit of " +
                                 std::to_string(kMaxGrid) + " grid points");
  if (c->wires[w].nr > kMaxNr)
    return fail(SBE_ERR_UNSUPPORTED, "sbe_prop2qw_noalloc: wire Nr = " +
                                         std::to_string(c->wires[w].nr) +
                                         " exceeds the static scratch limit of " +
                                         std::to_string(kMaxNr) + " (Nk <= 1024)");
  double2* scratch = nullptr;
  int rc = scratch_ptr(&scratch);
  if (rc) return rc;
  return launch_prop2qw_scratch(c, w, RR, n_rr, reinterpret_cast<const double2*>(fields_in),
                                reinterpret_cast<double2*>(out), scratch, scratch + kCoefElems,
                                as_stream(stream));
}
