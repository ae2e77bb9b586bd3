// Batched strided complex FFT passes for the oversampled 3D grid (the algorithm and the
// kernels are in fft_kernels.cuh).  This unit holds the twiddle tables, the dispatch and
// the kernels for lines of 16..160 points and the lengths with a prime factor >= 7;
// fft_large.cu and fft_large2.cu instantiate the other longer lines, so the three compile
// in parallel.
#include "fft_kernels.cuh"

namespace mrg {

// line lengths S = 8 Q; the default oversampled size 16 ceil(1.5 N / 16) is 8 Q with Q
// even, so every N up to 256 has its length here
static const int kSupportedQ[] = {2,  3,  4,  5,  6,  8,  9,  10, 12, 14, 15, 16, 18, 20, 22, 24, 26,
                                  28, 30, 32, 34, 36, 38, 40, 42, 44, 45, 46, 48};
// lines of 400..768 points: S = 16 Q (fft_long.cu)
static const int kLongQ[] = {25, 26, 27, 28, 30, 32, 33, 34, 35, 36, 38, 39, 40, 42, 44, 45, 46, 48};

bool fft_size_supported(int S) {
  if (S % 8) return false;
  for (int q : kSupportedQ)
    if (q * 8 == S) return true;
  for (int q : kLongQ)
    if (q * 16 == S) return true;
  return false;
}

int fft_max_lines_per_cta(int S) { return S > 384 ? 16 : 32; }

// Per-size twiddle tables exp(-2 pi i m / S), m < S, built once on each device (a table
// lives in the memory of the device it was built on).
static float2 *g_tw[kTwDevices][1024];
static DeviceOnce g_tw_once;

mrg_status fft_init_device() {
  int dev = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kTwDevices) {
    set_error("device ordinal beyond the FFT twiddle tables");
    return MRG_ERR_UNSUPPORTED;
  }
  return device_once(g_tw_once, [dev]() -> mrg_status {
    std::vector<int> sizes;
    for (int q : kSupportedQ) sizes.push_back(8 * q);
    for (int q : kLongQ) sizes.push_back(16 * q);
    for (int S : sizes) {
      std::vector<float2> tw(S);
      for (int m = 0; m < S; m++) {
        const double a = -2.0 * 3.141592653589793238462643 * (double)m / (double)S;
        tw[m] = make_float2((float)cos(a), (float)sin(a));
      }
      MRG_CUDA(cudaMalloc(&g_tw[dev][S], sizeof(float2) * S));
      MRG_CUDA(cudaMemcpy(g_tw[dev][S], tw.data(), sizeof(float2) * S, cudaMemcpyHostToDevice));
    }
    return MRG_OK;
  });
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    else
      cudaGetLastError();
  });
  return fn;
}

const float2 *fft_twiddles(int S) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kTwDevices || S < 0 || S >= 1024) return nullptr;
  return g_tw[dev][S];
}


void fft_vectorize(FftPass &p) {
  auto al = [](const void *q) { return ((uintptr_t)q & 15) == 0; };
  const bool pairs = !p.lfast && (p.IB % 2 == 0) && (p.inner % 2 == 0) && (p.nlines % 2 == 0);
  const float2 *src = (p.mode == FFT_SETIMG) ? p.smap : p.in;
  p.vec16 = pairs && src && al(src) && (p.in_os % 2 == 0) && (p.in_ls % 2 == 0);
  p.vec16o = pairs && p.mode != FFT_ACCUM && p.out && al(p.out) && (p.out_os % 2 == 0) && (p.out_ls % 2 == 0);
}

mrg_status launch_fft(const FftPass &p, cudaStream_t st) {
  if (p.nlines <= 0) return MRG_OK;
  if ((p.mode == FFT_SETIMG && p.sign >= 0) || (p.mode == FFT_ACCUM && p.sign <= 0)) {
    set_error("fft pass: mode/sign mismatch");
    return MRG_ERR_INVALID;
  }
  if (p.IB < 1 || p.IB > 32) {
    set_error("fft pass: bad IB");
    return MRG_ERR_INVALID;
  }
  if ((p.vec16 || p.vec16o) && (p.lfast || (p.IB & 1))) {
    set_error("fft pass: 16-byte copies need paired lines");
    return MRG_ERR_INVALID;
  }
  if (p.lfast && (p.mode != FFT_PLAIN || p.inner != 1)) {
    set_error("fft pass: contiguous-line mode needs a plain pass over single lines");
    return MRG_ERR_INVALID;
  }
  switch (p.S) {
    case 16: return launch_q<2>(p, st);
    case 24: return launch_q<3>(p, st);
    case 32: return launch_q<4>(p, st);
    case 40: return launch_q<5>(p, st);
    case 48: return launch_q<6>(p, st);
    case 64: return launch_q<8>(p, st);
    case 72: return launch_q<9>(p, st);
    case 80: return launch_q<10>(p, st);
    case 96: return launch_q<12>(p, st);
    case 120: return launch_q<15>(p, st);
    case 128: return launch_q<16>(p, st);
    case 144: return launch_q<18>(p, st);
    case 160: return launch_q<20>(p, st);
    case 112: return launch_q<14>(p, st);
    case 176: return launch_q<22>(p, st);
    case 208: return launch_q<26>(p, st);
    case 224: return launch_q<28>(p, st);
    case 272: return launch_q<34>(p, st);
    case 304: return launch_q<38>(p, st);
    case 192:
    case 240:
    case 256:
    case 288: return launch_fft_192_288(p, st);
    case 336: return launch_q<42>(p, st);
    case 352: return launch_q<44>(p, st);
    case 368: return launch_q<46>(p, st);
    case 320:
    case 360:
    case 384: return launch_fft_320_384(p, st);
    default:
      if (p.S > 384) return launch_fft_long(p, st);
      set_error("unsupported FFT length " + std::to_string(p.S));
      return MRG_ERR_UNSUPPORTED;
  }
}

}  // namespace mrg
