// nrg_broaden_noalloc: the log-Gaussian broadening of nrg_broaden run on
// caller-owned device buffers, with its one intermediate array (ln e_i per
// bin) in a file-scope device array instead of an allocation.  Nothing here
// calls cudaMalloc, cudaMallocAsync, cudaFree or any allocating library
// routine; the entry point only launches k_log_energies and k_broaden.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "nrg_gpu.h"
#include "nrg_internal.h"

namespace nrg {
extern thread_local std::string g_err;
}

// ln(e_i) of every bin of one call (NaN for zero-weight bins, which the
// broadening then skips).  No entry has to start at zero: each call writes
// entries [0, nbins) before k_broaden reads them.
static __device__ __align__(256) double g_broaden_lnE[NRG_BROADEN_NOALLOC_MAX_BINS];

namespace {

__global__ void k_log_energies(const double *__restrict__ e, const double *__restrict__ w, int64_t n,
                               double *__restrict__ le) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    le[i] = (w[i] != 0.0) ? log(e[i]) : __longlong_as_double(0x7ff8000000000000LL);
}

struct Fail {
  int code;
  std::string msg;
};

// Device address of the scratch on the current device.  Looked up with the
// caller's device current on every call rather than cached: after a
// cudaDeviceReset (or any re-creation of the primary context) the module is
// loaded again and the array may move, so a cached address could point at
// freed memory.  Once the module is loaded the lookup is a table search.
double *scratch_for_current_device() {
  void *p = nullptr;
  const cudaError_t rc = cudaGetSymbolAddress(&p, g_broaden_lnE);
  if (rc == cudaErrorNoDevice || rc == cudaErrorInsufficientDriver)
    throw Fail{NRG_E_NOCUDA, std::string("cudaGetSymbolAddress(broaden scratch): ") + cudaGetErrorString(rc)};
  if (rc != cudaSuccess || !p)
    throw Fail{NRG_E_CUDA, std::string("cudaGetSymbolAddress(broaden scratch): ") + cudaGetErrorString(rc)};
  return static_cast<double *>(p);
}

}  // namespace

extern "C" int nrg_broaden_noalloc(const double *energies, const double *weights, uint64_t nbins,
                                   const double *omegas, uint64_t nomega, double b, double *out,
                                   void *stream) {
  try {
    if (nbins > uint64_t(NRG_BROADEN_NOALLOC_MAX_BINS))
      throw Fail{NRG_E_ARG, "nrg_broaden_noalloc: nbins = " + std::to_string(nbins) +
                                " exceeds the static scratch of " +
                                std::to_string(NRG_BROADEN_NOALLOC_MAX_BINS) + " bins"};
    if (nomega > uint64_t(0x7fffffff))
      throw Fail{NRG_E_ARG, "nrg_broaden_noalloc: nomega = " + std::to_string(nomega) +
                                " exceeds one launch (2^31 - 1 frequencies)"};
    if ((nbins && (!energies || !weights)) || (nomega && (!omegas || !out)))
      throw Fail{NRG_E_ARG, "nrg_broaden_noalloc: null device pointer"};
    if (!(b > 0.0)) throw Fail{NRG_E_ARG, "nrg_broaden_noalloc: broadening width b must be > 0"};
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *le = scratch_for_current_device();
    if (nbins) {
      int grid = int((nbins + 255) / 256);
      if (grid > 152 * 8) grid = 152 * 8;
      k_log_energies<<<grid, 256, 0, s>>>(energies, weights, int64_t(nbins), le);
    }
    nrg::launch_broaden(le, weights, int64_t(nbins), omegas, int64_t(nomega), b, out, s);
    const cudaError_t rc = cudaGetLastError();
    if (rc != cudaSuccess) throw Fail{NRG_E_CUDA, std::string("nrg_broaden_noalloc launch: ") + cudaGetErrorString(rc)};
    return NRG_OK;
  } catch (const Fail &f) {
    nrg::g_err = f.msg;
    return f.code;
  }
}
