// Low-rank threshold estimate that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a reconstruction service that reserves its
// whole GPU memory budget at start-up (or shares the process with a caching
// allocator that already holds it) has nothing left for a per-call allocation, and
// a streamed pipeline cannot afford the device-wide synchronisation that
// cudaMalloc / cudaFree may cause between its kernels.  For them this entry point
// keeps its scratch -- the largest singular value of every block and the buffer of
// the median's sort -- in a fixed file-scope device array, sized for at most
// MRG_NOALLOC_MAX_BLOCKS blocks (512 KiB, held by every GPU that loads the library
// until the process exits).
#include <mutex>

#include "mrg_internal.h"

using namespace mrg;

namespace {

// sigma_1 per block [0, MAX), then the sort buffer [MAX, 2*MAX), then smax (as bits).
__device__ __align__(256) double g_llr_scratch[2 * MRG_NOALLOC_MAX_BLOCKS + 1];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device, looked up once per
// device with that device current.
mrg_status scratch_address(double **out) {
  int dev = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal out of range for the no-allocation scratch table");
    return MRG_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_llr_scratch);
    if (e != cudaSuccess) {
      set_error(std::string("cudaGetSymbolAddress(g_llr_scratch) failed: ") + cudaGetErrorString(e));
      return MRG_ERR_CUDA;
    }
    g_scratch[dev] = static_cast<double *>(p);
  }
  *out = g_scratch[dev];
  return MRG_OK;
}

bool on_device(const void *ptr) {
  cudaPointerAttributes a;
  if (!ptr || cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" mrg_status mrg_llr_update_threshold_noalloc(const void *X, int nframes, int Nx, int Ny, int Nz,
                                                       const int block[3], float clear_amp, float clear_t2,
                                                       int iteration, float *smax, void *stream) {
  if (!X || !block || !smax || nframes <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || block[0] <= 0 || block[1] <= 0 ||
      block[2] <= 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  if (!on_device(X)) {
    set_error("mrg_llr_update_threshold_noalloc needs X in device memory (staging a host copy would allocate)");
    return MRG_ERR_INVALID;
  }
  const int N[3] = {Nx, Ny, Nz};
  const int64_t nb = llr_block_count(N, block);  // 64-bit: a huge shape cannot wrap under the limit
  if (nb > MRG_NOALLOC_MAX_BLOCKS) {
    set_error("mrg_llr_update_threshold_noalloc: " + std::to_string(nb) + " low-rank blocks exceed the limit of " +
              std::to_string(MRG_NOALLOC_MAX_BLOCKS) + " of its fixed scratch array");
    return MRG_ERR_UNSUPPORTED;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const bool smax_on_device = on_device(smax);
  if (!smax_on_device) {
    // a host smax is read back with a stream synchronisation, which a capturing stream forbids
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    MRG_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) {
      set_error("mrg_llr_update_threshold_noalloc inside a stream capture needs smax in device memory");
      return MRG_ERR_INVALID;
    }
  }
  double *scratch = nullptr;
  MRG_TRY(scratch_address(&scratch));
  float *smax_dev = reinterpret_cast<float *>(scratch + 2 * MRG_NOALLOC_MAX_BLOCKS);
  // every scratch element the kernels read is written first in this call: no clearing needed
  MRG_TRY(llr_update_into(static_cast<const float2 *>(X), nframes, N, block, clear_amp, clear_t2, nullptr, iteration,
                          scratch, scratch + MRG_NOALLOC_MAX_BLOCKS, smax_dev, st));
  MRG_CUDA(cudaMemcpyAsync(smax, smax_dev, sizeof(float), cudaMemcpyDefault, st));
  if (!smax_on_device) MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}
