// Coil images, sum-of-squares images and the low-resolution coil-map estimate.
//
// gridFFT::forward without a map (src/gridFFT.cpp:759-789) ends with
// accumulate(X) (:943-958): X += winz*winy*winx * image, one image per coil.
// gridFFT::forward_sos (:722-757) ends with deapp (:912-924) and
// accumulate_sos (:960-970): X += |win * image|^2, summed over the coils by the
// caller.  The E^H passes up to the cropped z transform are the shared ones;
// the kernels here replace its epilogue, reading the transformed crop
// t[z][y][x][c] (coils innermost).
//
// The map estimate (RECON::..., src/recon_lib.cpp:2694-2950, LOWRES branch
// with SOS normalisation) grids each coil with k_rad lowered to the map
// resolution, blurs the images (gaussian_blur_template,
// src/ArrayTemplates.cpp:489-601) and divides every coil by the root sum of
// squares over coils (RECON::sos_normalize, src/recon_lib.cpp:3043-3062).
#include "mrg_internal.h"

namespace mrg {

// Deapodisation weight of voxel (x, y, z): (winz * winy) * winx in float, the
// reference's order.  wx/wy/wz already point at the crop start.
__device__ __forceinline__ float deapod(const float *wx, const float *wy, const float *wz, int x, int y, int z) {
  return __fmul_rn(__fmul_rn(wz[z], wy[y]), wx[x]);
}

// out[c * vs + v * es] (+)= w(v) * t[v][c]
__global__ void k_coil_images(const float2 *__restrict__ t, int C, int Nx, int Ny, int64_t nimg,
                              const float *__restrict__ wx, const float *__restrict__ wy, const float *__restrict__ wz,
                              float2 *out, int64_t es, int64_t vs, int accumulate, int coil_major) {
  const int64_t n = nimg * C;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t v;
    int c;
    if (coil_major) {  // consecutive threads write consecutive voxels of one coil
      c = (int)(idx / nimg);
      v = idx - (int64_t)c * nimg;
    } else {
      v = idx / C;
      c = (int)(idx - v * C);
    }
    const int x = (int)(v % Nx), y = (int)((v / Nx) % Ny), z = (int)(v / ((int64_t)Nx * Ny));
    const float w = deapod(wx, wy, wz, x, y, z);
    const float2 a = t[v * C + c];
    const float2 r = make_float2(__fmul_rn(w, a.x), __fmul_rn(w, a.y));
    float2 *d = out + (int64_t)c * vs + v * es;
    if (accumulate) {
      const float2 o = *d;
      *d = make_float2(__fadd_rn(o.x, r.x), __fadd_rn(o.y, r.y));
    } else {
      *d = r;
    }
  }
}

// X[v] += sum_c |w(v) * t[v][c]|^2, added coil by coil as the reference's loop does.
__global__ void k_sos_images(const float2 *__restrict__ t, int C, int Nx, int Ny, int64_t nimg,
                             const float *__restrict__ wx, const float *__restrict__ wy, const float *__restrict__ wz,
                             float2 *X) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nimg; v += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(v % Nx), y = (int)((v / Nx) % Ny), z = (int)(v / ((int64_t)Nx * Ny));
    const float w = deapod(wx, wy, wz, x, y, z);
    float2 acc = X[v];
    for (int c = 0; c < C; c++) {
      const float2 a = t[v * C + c];
      const float re = __fmul_rn(a.x, w), im = __fmul_rn(a.y, w);
      acc.x = __fadd_rn(acc.x, __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im)));
    }
    X[v] = acc;
  }
}

mrg_status launch_coil_images(const float2 *t, int C, const int N[3], const float *wx, const float *wy,
                              const float *wz, float2 *out, int64_t es, int64_t vs, bool accumulate,
                              cudaStream_t st) {
  const int64_t nimg = (int64_t)N[0] * N[1] * N[2];
  const int coil_major = (es == 1) ? 1 : 0;
  k_coil_images<<<grid_blocks(nimg * C, 256), 256, 0, st>>>(t, C, N[0], N[1], nimg, wx, wy, wz, out, es, vs,
                                                            accumulate ? 1 : 0, coil_major);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status launch_sos_images(const float2 *t, int C, const int N[3], const float *wx, const float *wy,
                             const float *wz, float2 *X, cudaStream_t st) {
  const int64_t nimg = (int64_t)N[0] * N[1] * N[2];
  k_sos_images<<<grid_blocks(nimg, 256), 256, 0, st>>>(t, C, N[0], N[1], nimg, wx, wy, wz, X);
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// Gaussian blur along one axis.  A CTA stages 32 lines in shared memory
// ([n][33] complex) and writes every output point of them:
//   out[i] = sum_{ii = max(i - w, 0)}^{min(i + w, n) - 1} kern[ii - i + w] * in[ii]
// (the reference's loop bound excludes ii = i + w).
// Lines are enumerated over three outer dimensions ordered by stride, so the
// 32 lines of a CTA are as close in memory as the layout allows.
// ---------------------------------------------------------------------------
constexpr int MAX_BLUR_TAPS = 255;

struct BlurArgs {
  float2 *X;
  int n;             // line length
  int64_t ls;        // element stride along the line
  int64_t on[3];     // outer sizes, fastest first
  int64_t os[3];     // outer strides
  int64_t nlines;
  int w;             // half width
  float kern[MAX_BLUR_TAPS];
};

__global__ void __launch_bounds__(256) k_blur(const BlurArgs a) {
  extern __shared__ float2 bsm[];  // [n][33]
  const float *kern = a.kern;
  const int64_t l0 = (int64_t)blockIdx.x * 32;
  const bool lfast = (a.ls == 1);
  for (int e = threadIdx.x; e < 32 * a.n; e += blockDim.x) {
    const int jj = lfast ? e / a.n : e % 32;
    const int r = lfast ? e % a.n : e / 32;
    const int64_t l = l0 + jj;
    if (l < a.nlines) {
      const int64_t i0 = l % a.on[0], i1 = (l / a.on[0]) % a.on[1], i2 = l / (a.on[0] * a.on[1]);
      bsm[r * 33 + jj] = a.X[i0 * a.os[0] + i1 * a.os[1] + i2 * a.os[2] + r * a.ls];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * a.n; e += blockDim.x) {
    const int jj = lfast ? e / a.n : e % 32;
    const int i = lfast ? e % a.n : e / 32;
    const int64_t l = l0 + jj;
    if (l >= a.nlines) continue;
    const int s0 = max(i - a.w, 0), e0 = min(i + a.w, a.n);
    float2 acc = make_float2(0.f, 0.f);
    for (int ii = s0; ii < e0; ii++) {
      const float k = kern[ii - (i - a.w)];
      const float2 v = bsm[ii * 33 + jj];
      acc.x = __fadd_rn(acc.x, __fmul_rn(k, v.x));
      acc.y = __fadd_rn(acc.y, __fmul_rn(k, v.y));
    }
    const int64_t i0 = l % a.on[0], i1 = (l / a.on[0]) % a.on[1], i2 = l / (a.on[0] * a.on[1]);
    a.X[i0 * a.os[0] + i1 * a.os[1] + i2 * a.os[2] + (int64_t)i * a.ls] = acc;
  }
}

// Kernel taps of one axis on the host, as gaussian_blur_template builds them:
// kern[t] = exp(-((float)t - w)^2 / (2.0 * sigma^2)), then kern /= sum(kern).
static void blur_kernel(float sigma, std::vector<float> &kern) {
  const int w = (int)(5 * sigma);
  kern.assign(2 * w + 1, 0.f);
  double tot = 0;
  for (int t = 0; t <= 2 * w; t++) {
    const float a = (float)t - w;
    kern[t] = (float)std::exp(-(a * a) / (2.0 * (double)(sigma * sigma)));
  }
  for (int t = 0; t <= 2 * w; t++) tot += kern[t];
  for (int t = 0; t <= 2 * w; t++) kern[t] = (float)(kern[t] / tot);
}

// Blur nvol volumes in place; element (x, y, z) of volume c is at
// X + c * vs + ((z * Ny + y) * Nx + x) * es.
mrg_status gaussian_blur_ex(float2 *X, int nvol, const int N[3], int64_t es, int64_t vs, const float sigma[3],
                            cudaStream_t st) {
  for (int d = 0; d < 3; d++) {
    if (!(sigma[d] > 0)) continue;
    std::vector<float> kern;
    blur_kernel(sigma[d], kern);
    const int w = (int)kern.size() / 2;
    const size_t smem = (size_t)N[d] * 33 * sizeof(float2);
    if (smem > 227 * 1024 || (int)kern.size() > MAX_BLUR_TAPS) {
      set_error("blur line or kernel too long for one CTA");
      return MRG_ERR_UNSUPPORTED;
    }
    BlurArgs a;
    for (int t = 0; t < (int)kern.size(); t++) a.kern[t] = kern[t];
    a.X = X;
    a.n = N[d];
    const int64_t axs[3] = {es, es * N[0], es * N[0] * N[1]};
    a.ls = axs[d];
    // outer dims: the two other axes and the volume index, sorted by stride
    int64_t sz[3] = {N[(d + 1) % 3], N[(d + 2) % 3], nvol};
    int64_t sd[3] = {axs[(d + 1) % 3], axs[(d + 2) % 3], vs};
    for (int i = 0; i < 3; i++)
      for (int j = i + 1; j < 3; j++)
        if (sd[j] < sd[i]) {
          std::swap(sd[i], sd[j]);
          std::swap(sz[i], sz[j]);
        }
    for (int i = 0; i < 3; i++) {
      a.on[i] = sz[i];
      a.os[i] = sd[i];
    }
    a.nlines = sz[0] * sz[1] * sz[2];
    a.w = w;
    static DeviceOnce once;
    MRG_TRY(device_once(once, []() -> mrg_status {
      MRG_CUDA(cudaFuncSetAttribute(k_blur, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
      return MRG_OK;
    }));
    k_blur<<<(unsigned)((a.nlines + 31) / 32), 256, smem, st>>>(a);
    MRG_LAUNCHED();
  }
  return MRG_OK;
}

// A[c * vs + v * es] /= sqrt(sum_c |A_c(v)|^2), the sum taken coil by coil in float.
__global__ void k_sos_normalize(float2 *A, int C, int64_t nimg, int64_t es, int64_t vs) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nimg; v += (int64_t)gridDim.x * blockDim.x) {
    float sos = 0.f;
    for (int c = 0; c < C; c++) {
      const float2 a = A[c * vs + v * es];
      sos = __fadd_rn(sos, __fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)));
    }
    sos = __fsqrt_rn(sos);
    for (int c = 0; c < C; c++) {
      float2 *p = A + c * vs + v * es;
      const float2 a = *p;
      *p = make_float2(__fdiv_rn(a.x, sos), __fdiv_rn(a.y, sos));
    }
  }
}

mrg_status sos_normalize_ex(float2 *A, int C, int64_t nimg, int64_t es, int64_t vs, cudaStream_t st) {
  k_sos_normalize<<<grid_blocks(nimg, 256), 256, 0, st>>>(A, C, nimg, es, vs);
  MRG_LAUNCHED();
  return MRG_OK;
}

}  // namespace mrg
