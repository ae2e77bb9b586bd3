// FFT passes for lines of 320, 360, 384 points (kernels in fft_kernels.cuh).
#include "fft_kernels.cuh"

namespace mrg {

mrg_status launch_fft_320_384(const FftPass &p, cudaStream_t st) {
  switch (p.S) {
    case 320: return launch_q<40>(p, st);
    case 360: return launch_q<45>(p, st);
    case 384: return launch_q<48>(p, st);
    default:
      set_error("unsupported FFT length " + std::to_string(p.S));
      return MRG_ERR_UNSUPPORTED;
  }
}

}  // namespace mrg
