// Fraction thresholding (THRESHOLD::get_threshold, src/threshold.cpp:251-391)
// and complex soft thresholding (src/threshold.cpp:766-814).
//
// The bisection is a fixed sequence of at most 64 counting rounds whose
// decisions stay on the device: a one-thread step kernel updates the bracket
// from the previous count and sets `done` when the reference's loop would stop;
// the counting kernels of later rounds then return at once.  No round trip to
// the host, so the whole update can sit inside a captured FISTA iteration.
// |c| is formed as sqrt(re^2 + im^2) in double and rounded once, as glibc's
// hypotf does for std::abs(complex<float>).
#include "mrg_internal.h"

namespace mrg {

struct ThrState {
  float value, min_t, max_t, mx, mn;
  int done, iter, pad;
  long long found, target, acc, count, total;
};

__device__ __forceinline__ float cabs_ref(float2 c) {
  return (float)sqrt((double)c.x * (double)c.x + (double)c.y * (double)c.y);
}

__global__ void k_thr_reset(ThrState *s, int64_t n) {
  s->mx = 0.0f;
  s->mn = __int_as_float(0x7f800000);
  s->done = 0;
  s->iter = 0;
  s->count = 0;
  s->total = n;
}

__global__ void k_thr_mag(const float2 *__restrict__ X, int64_t n, float *mag, ThrState *s) {
  float mx = 0.0f, mn = __int_as_float(0x7f800000);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float a = cabs_ref(X[i]);
    mag[i] = a;
    mx = fmaxf(mx, a);
    mn = fminf(mn, a);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
  }
  if ((threadIdx.x & 31) == 0) {
    // non-negative floats order like their bit patterns
    atomicMax((int *)&s->mx, __float_as_int(mx));
    atomicMin((int *)&s->mn, __float_as_int(mn));
  }
}

__global__ void k_thr_init(ThrState *s, float fraction) {
  const long long total = s->total;
  s->target = (long long)(fraction * (double)total);
  s->acc = (long long)(0.001 * (double)total);
  s->found = total;
  s->iter = 0;
  if (s->target < 2) {
    s->value = 0.0f;
    s->done = 1;
    return;
  }
  s->value = (float)(0.5 * (s->mx - s->mn));
  s->max_t = (float)((double)fraction * s->mx);
  s->min_t = s->mn;
}

__global__ void k_thr_step(ThrState *s) {
  if (s->done) return;
  if (s->iter > 0) s->found = s->count;
  long long d = s->found - s->target;
  if (d < 0) d = -d;
  if (!(d > s->acc && s->iter < 64)) {
    s->done = 1;
    return;
  }
  if (s->iter > 0) {
    if (s->found > s->target) s->max_t = s->value;
    else s->min_t = s->value;
    s->value = (float)(0.5 * (s->max_t + s->min_t));
  }
  s->iter += 1;
  s->count = 0;
}

__global__ void k_thr_count(const float *__restrict__ mag, int64_t n, ThrState *s) {
  if (s->done) return;
  const float v = s->value;
  long long c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += (mag[i] < v) ? 1 : 0;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd((unsigned long long *)&s->count, (unsigned long long)c);
}

__global__ void k_thr_finish(const ThrState *s, float scale, float *out) { *out = scale * s->value; }

mrg_status thr_alloc(ThrWork &w, int64_t n) {
  if (w.cap >= n && w.mag) return MRG_OK;
  thr_free(w);
  MRG_CUDA(cudaMalloc(&w.mag, sizeof(float) * (size_t)std::max<int64_t>(n, 1)));
  MRG_CUDA(cudaMalloc(&w.state, sizeof(ThrState)));
  w.cap = n;
  return MRG_OK;
}

void thr_free(ThrWork &w) {
  cudaFree(w.mag);
  cudaFree(w.state);
  w.mag = nullptr;
  w.state = nullptr;
  w.cap = 0;
}

static int thr_blocks(int64_t n) {
  int64_t b = (n + 1023) / 1024;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 8));
}

mrg_status fraction_threshold(const float2 *X, int64_t n, float fraction, float scale, ThrWork &w, float *out_dev,
                              cudaStream_t st) {
  ThrState *s = (ThrState *)w.state;
  const int nb = thr_blocks(n);
  k_thr_reset<<<1, 1, 0, st>>>(s, n);
  MRG_LAUNCHED();
  k_thr_mag<<<nb, 256, 0, st>>>(X, n, w.mag, s);
  MRG_LAUNCHED();
  k_thr_init<<<1, 1, 0, st>>>(s, fraction);
  MRG_LAUNCHED();
  for (int r = 0; r < 64; r++) {
    k_thr_step<<<1, 1, 0, st>>>(s);
    MRG_LAUNCHED();
    k_thr_count<<<nb, 256, 0, st>>>(w.mag, n, s);
    MRG_LAUNCHED();
  }
  k_thr_step<<<1, 1, 0, st>>>(s);
  MRG_LAUNCHED();
  k_thr_finish<<<1, 1, 0, st>>>(s, scale, out_dev);
  MRG_LAUNCHED();
  return MRG_OK;
}

__global__ void k_soft(float2 *__restrict__ X, int64_t n, const float *__restrict__ value) {
  const float v = *value;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 c = X[i];
    const float cc = cabs_ref(c);
    if (cc <= v) {
      X[i] = make_float2(0.f, 0.f);
    } else {
      const float f = 1.0f - v / cc;
      X[i] = make_float2(c.x * f, c.y * f);
    }
  }
}

mrg_status soft_threshold(float2 *X, int64_t n, const float *value_dev, cudaStream_t st) {
  k_soft<<<thr_blocks(n), 256, 0, st>>>(X, n, value_dev);
  MRG_LAUNCHED();
  return MRG_OK;
}

}  // namespace mrg
