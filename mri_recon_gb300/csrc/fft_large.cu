// FFT passes for lines of 192, 240, 256, 288 points (kernels in fft_kernels.cuh).
#include "fft_kernels.cuh"

namespace mrg {

mrg_status launch_fft_192_288(const FftPass &p, cudaStream_t st) {
  switch (p.S) {
    case 192: return launch_q<24>(p, st);
    case 240: return launch_q<30>(p, st);
    case 256: return launch_q<32>(p, st);
    case 288: return launch_q<36>(p, st);
    default:
      set_error("unsupported FFT length " + std::to_string(p.S));
      return MRG_ERR_UNSUPPORTED;
  }
}

}  // namespace mrg
