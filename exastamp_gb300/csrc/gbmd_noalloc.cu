// gbmd_noalloc.cu -- the thermodynamic reduction for callers that may not
// allocate device memory.
//
// gbmd_thermo() keeps its per-block partial sums in a buffer the context
// allocates.  Some callers cannot allow that: a plugin running inside a host
// framework whose device memory all comes from the framework's own pool, a
// caller in the middle of capturing a CUDA graph on its stream (cudaMalloc
// is not stream-ordered and may synchronise the device), or a
// latency-critical loop where a device-wide synchronisation is not
// acceptable.  gbmd_thermo_reduce_noalloc() runs the same two reduction
// kernels on the caller's device arrays and uses, as scratch, a fixed array
// in this library's own device image instead of an allocation.
#include "gbmd_internal.cuh"

namespace {

// One row of 26 partial sums per reduction block.  The reduction never uses
// more than TH_MAX_BLOCKS blocks, so the scratch is TH_MAX_BLOCKS x 26
// doubles (1184 x 26 = 246,272 bytes) on every device that loads the
// library, held until the process exits.
constexpr int kScratchRows = gbmd::TH_MAX_BLOCKS;
static_assert(kScratchRows >= gbmd::TH_MAX_BLOCKS, "thermo scratch smaller than the reduction grid");

static __device__ __align__(256) double g_thermo_scratch[kScratchRows * 26];

// Device address of the scratch array in the current device's context.  It
// is looked up on every call (a host-side table lookup that allocates
// nothing), so it stays right when the context has been torn down and
// re-created in between, e.g. after cudaDeviceReset, where a cached address
// would point into the old module.
int scratch_for_current_device(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_thermo_scratch);
  if (e != cudaSuccess || !p) return GBMD_ERR_CUDA;
  *out = static_cast<double*>(p);
  return GBMD_OK;
}

}  // namespace

extern "C" int gbmd_thermo_reduce_noalloc(int64_t n, const double* vx, const double* vy, const double* vz,
                                          const double* ep, const double* vir, const uint8_t* type,
                                          const double* masses, int ntypes, double* out, void* stream) {
  if (n < 0) return GBMD_ERR_INVALID;
  if (n > GBMD_MAX_ATOMS) return GBMD_ERR_TOO_LARGE;
  if (ntypes < 1 || ntypes > GBMD_MAX_TYPES || !masses || !out) return GBMD_ERR_INVALID;
  if (n > 0 && (!vx || !vy || !vz || !type)) return GBMD_ERR_INVALID;
  double* scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch);
  if (rc != GBMD_OK) return rc;
  gbmd::launch_thermo_raw(n, vx, vy, vz, ep, vir, type, masses, ntypes, scratch, out,
                          static_cast<cudaStream_t>(stream));
  return cudaGetLastError() == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}
