// Separable periodic 3D wavelet with circular shifts (WAVELET3D,
// src/wavelet3D.cpp:563-791).
//
// One pass transforms every line of one axis inside the current sub-box
// [0,Lx) x [0,Ly) x [0,Lz) of each volume.  A CTA stages 32 lines in shared
// memory and computes each output position as a gather:
//   analysis  out[p]       = sum_f lpf[f] * in[(2p - f + S) mod L]      (p < L/2)
//             out[p + L/2] = sum_f hpf[f] * in[(2p - f + S) mod L]
//   synthesis out[c] = sum_f [in[p] Slpf[f] + in[p + L/2] Shpf[f]] over the
//             f with 2p = c - f + wN - 1 - S (mod L), the transpose of
//             iwave1D's scatter (wavelet3D.cpp:775-791).
// The shift S of each axis is read from device memory (indexed by the
// iteration counter when a whole FISTA iteration is replayed from a graph).
#include "mrg_internal.h"

namespace mrg {

struct WaveFilt {
  float lpf[4], hpf[4], slpf[4], shpf[4];
  int wN;
};

struct WaveArgs {
  float2 *X;
  int64_t vstride;
  int Nx, Ny;
  int axis, L, Lx, Ly, Lz;
  int64_t nlines;
  WaveFilt f;
  const int *shifts;      // shift table
  const Scalars *sc;      // iteration counter (may be NULL)
  int per_it, off;        // shift = shifts[(sc ? sc->it : 0) * per_it + off + axis]
};

static WaveFilt filters(int type) {
  WaveFilt f;
  if (type == 0) {  // DB2 / Haar (wavelet3D.cpp:122-140)
    const float h = (float)(1.0 / std::sqrt(2.0));
    f.wN = 2;
    f.lpf[0] = h; f.lpf[1] = h; f.hpf[0] = -h; f.hpf[1] = h;
    f.slpf[0] = h; f.slpf[1] = h; f.shpf[0] = h; f.shpf[1] = -h;
    for (int k = 2; k < 4; k++) f.lpf[k] = f.hpf[k] = f.slpf[k] = f.shpf[k] = 0.f;
  } else {  // Daubechies-4 from its closed form, arranged as wavelet3D.cpp:168-186
    const double s3 = std::sqrt(3.0), d = 4.0 * std::sqrt(2.0);
    const double h0 = (1 + s3) / d, h1 = (3 + s3) / d, h2 = (3 - s3) / d, h3 = (1 - s3) / d;
    f.wN = 4;
    f.lpf[0] = (float)h3; f.lpf[1] = (float)h2; f.lpf[2] = (float)h1; f.lpf[3] = (float)h0;
    f.hpf[0] = (float)-h0; f.hpf[1] = (float)h1; f.hpf[2] = (float)-h2; f.hpf[3] = (float)h3;
    f.slpf[0] = (float)h0; f.slpf[1] = (float)h1; f.slpf[2] = (float)h2; f.slpf[3] = (float)h3;
    f.shpf[0] = (float)h3; f.shpf[1] = (float)-h2; f.shpf[2] = (float)h1; f.shpf[3] = (float)-h0;
  }
  return f;
}

__device__ __forceinline__ int64_t wave_base(const WaveArgs &a, int64_t id, int64_t &stride) {
  if (a.axis == 0) {
    const int64_t y = id % a.Ly, z = id / a.Ly;
    stride = 1;
    return (z * a.Ny + y) * a.Nx;
  } else if (a.axis == 1) {
    const int64_t x = id % a.Lx, z = id / a.Lx;
    stride = a.Nx;
    return z * (int64_t)a.Nx * a.Ny + x;
  } else {
    const int64_t x = id % a.Lx, y = id / a.Lx;
    stride = (int64_t)a.Nx * a.Ny;
    return y * a.Nx + x;
  }
}

template <int INV>
__global__ void __launch_bounds__(256) k_wave(const WaveArgs a) {
  extern __shared__ float2 sm[];  // [L][33]
  __shared__ int64_t lbase[32];   // first element of each of the CTA's lines
  float2 *X = a.X + (int64_t)blockIdx.y * a.vstride;
  const int L = a.L, h = L / 2, wN = a.f.wN;
  // the shift taken modulo L once, so every index below wraps with one add or subtract
  int S = a.shifts[(a.sc ? a.sc->it : 0) * a.per_it + a.off + a.axis] % L;
  if (S < 0) S += L;
  const int64_t line0 = (int64_t)blockIdx.x * 32;
  const int nl = (int)min((int64_t)32, a.nlines - line0);  // lines of this CTA
  const bool lfast = (a.axis == 0);
  int64_t st = 1;
  wave_base(a, 0, st);  // the axis stride
  if (threadIdx.x < nl) {
    int64_t s2;
    lbase[threadIdx.x] = wave_base(a, line0 + threadIdx.x, s2);
  }
  __syncthreads();
  // load
  for (int e = threadIdx.x; e < 32 * L; e += blockDim.x) {
    const int jj = lfast ? e / L : (e & 31);
    const int l = lfast ? e - jj * L : (e >> 5);
    if (jj < nl) sm[l * 33 + jj] = X[lbase[jj] + l * st];
  }
  __syncthreads();
  // compute + store in place
  for (int e = threadIdx.x; e < 32 * L; e += blockDim.x) {
    const int jj = lfast ? e / L : (e & 31);
    const int o = lfast ? e - jj * L : (e >> 5);
    if (jj >= nl) continue;
    float2 acc = make_float2(0.f, 0.f);
    if (!INV) {
      const int p = (o < h) ? o : o - h;
      const float *flt = (o < h) ? a.f.lpf : a.f.hpf;
      for (int f = 0; f < wN; f++) {
        int c = 2 * p - f + S;  // in [-3, 2L - 1): (2p - f + S) mod L, a few steps at most
        while (c < 0) c += L;
        while (c >= L) c -= L;
        const float2 v = sm[c * 33 + jj];
        acc.x += flt[f] * v.x;
        acc.y += flt[f] * v.y;
      }
    } else {
      for (int f = 0; f < wN; f++) {
        int r = o - f + wN - 1 - S;  // in (-L, L + 3): (o - f + wN - 1 - S) mod L, a few steps at most
        while (r < 0) r += L;
        while (r >= L) r -= L;
        if (r & 1) continue;
        const int p = r >> 1;
        const float2 lo = sm[p * 33 + jj], hi = sm[(p + h) * 33 + jj];
        acc.x += lo.x * a.f.slpf[f];
        acc.y += lo.y * a.f.slpf[f];
        acc.x += hi.x * a.f.shpf[f];
        acc.y += hi.y * a.f.shpf[f];
      }
    }
    X[lbase[jj] + o * st] = acc;
  }
}

// Levels reduced until N / 2^L is an integer (wavelet3D.cpp:99-110).
void wavelet_levels(const int N[3], const int levels_in[3], int L[3], int *max_level) {
  *max_level = 0;
  for (int d = 0; d < 3; d++) {
    L[d] = levels_in[d];
    while (L[d] > 0 && (N[d] % (1 << L[d])) != 0) L[d]--;
    if (L[d] < 0) L[d] = 0;
    *max_level = std::max(*max_level, L[d]);
  }
}

static mrg_status wave_pass(WaveArgs a, int nvol, int inverse, cudaStream_t st) {
  a.L = a.axis == 0 ? a.Lx : (a.axis == 1 ? a.Ly : a.Lz);
  a.nlines = a.axis == 0 ? (int64_t)a.Ly * a.Lz : (a.axis == 1 ? (int64_t)a.Lx * a.Lz : (int64_t)a.Lx * a.Ly);
  if (a.L < 2 || a.nlines == 0) return MRG_OK;
  // dynamic shared memory: the staged lines; the kernel's own static 256 bytes (line bases)
  // come out of the same 227 KB per block
  constexpr int kDynMax = 227 * 1024 - 256;
  const size_t smem = (size_t)a.L * 33 * sizeof(float2);
  if (smem > (size_t)kDynMax) {
    set_error("wavelet line too long");
    return MRG_ERR_UNSUPPORTED;
  }
  const dim3 grid((unsigned)((a.nlines + 31) / 32), (unsigned)nvol);
  static DeviceOnce once;
  MRG_TRY(device_once(once, []() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_wave<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kDynMax));
    MRG_CUDA(cudaFuncSetAttribute(k_wave<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kDynMax));
    return MRG_OK;
  }));
  if (inverse) k_wave<1><<<grid, 256, smem, st>>>(a);
  else k_wave<0><<<grid, 256, smem, st>>>(a);
  MRG_LAUNCHED();
  return MRG_OK;
}

// forward3D / backward3D (wavelet3D.cpp:563-624) on nvol volumes.
mrg_status wavelet3d_ex(float2 *X, int nvol, const int N[3], const int L[3], int max_level, const int *shifts,
                        const Scalars *sc, int per_it, int off, int wave_type, int inverse, cudaStream_t st) {
  WaveArgs a;
  a.X = X;
  a.vstride = (int64_t)N[0] * N[1] * N[2];
  a.Nx = N[0];
  a.Ny = N[1];
  a.f = filters(wave_type);
  a.shifts = shifts;
  a.sc = sc;
  a.per_it = per_it;
  a.off = off;
  if (!inverse) {
    int sz = N[2], sy = N[1], sx = N[0];
    for (int l = 0; l < max_level; l++) {
      a.Lx = sx; a.Ly = sy; a.Lz = sz;
      if (l < L[0]) { a.axis = 0; MRG_TRY(wave_pass(a, nvol, 0, st)); }
      if (l < L[1]) { a.axis = 1; MRG_TRY(wave_pass(a, nvol, 0, st)); }
      if (l < L[2]) { a.axis = 2; MRG_TRY(wave_pass(a, nvol, 0, st)); }
      if (l < L[2]) sz = N[2] >> (l + 1);
      if (l < L[1]) sy = N[1] >> (l + 1);
      if (l < L[0]) sx = N[0] >> (l + 1);
    }
  } else {
    int sz = N[2] >> L[2], sy = N[1] >> L[1], sx = N[0] >> L[0];
    for (int l = max_level - 1; l >= 0; l--) {
      if (l < L[2]) sz = N[2] >> l;
      if (l < L[1]) sy = N[1] >> l;
      if (l < L[0]) sx = N[0] >> l;
      a.Lx = sx; a.Ly = sy; a.Lz = sz;
      if (l < L[2]) { a.axis = 2; MRG_TRY(wave_pass(a, nvol, 1, st)); }
      if (l < L[1]) { a.axis = 1; MRG_TRY(wave_pass(a, nvol, 1, st)); }
      if (l < L[0]) { a.axis = 0; MRG_TRY(wave_pass(a, nvol, 1, st)); }
    }
  }
  return MRG_OK;
}

mrg_status wavelet3d(float2 *X, int nvol, const int N[3], const int L[3], int max_level, const int *shifts_dev,
                     int wave_type, int inverse, cudaStream_t st) {
  return wavelet3d_ex(X, nvol, N, L, max_level, shifts_dev, nullptr, 0, 0, wave_type, inverse, st);
}

}  // namespace mrg
