// Image-domain vector kernels of the CG and FISTA loops.
//
// Vectors are complex64; inner products, residual norms and step sizes are
// accumulated and formed in FP64 on the device (src/recon_lib.cpp:1655-1722,
// :2072-2105), so a whole iteration runs without host round trips and can be
// captured in a CUDA graph.  Products are formed in float and then widened,
// as the reference does with norm(complex<float>) and conj(P)*LHS.
#include "mrg_internal.h"

namespace mrg {

constexpr int RT = 256;  // threads per reduction block

int reduce_blocks(int64_t n) {
  int64_t b = (n + RT * 8 - 1) / (RT * 8);
  if (b < 1) b = 1;
  if (b > 2048) b = 2048;
  return (int)b;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of NV doubles; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double red[NV][RT / 32];
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    v[k] = warp_sum(v[k]);
    if (l == 0) red[k][w] = v[k];
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      v[k] = (l < RT / 32) ? red[k][l] : 0.0;
      v[k] = warp_sum(v[k]);
    }
  }
}

__global__ void __launch_bounds__(RT) k_cg_dots(const float2 *__restrict__ R, const float2 *__restrict__ P,
                                               const float2 *__restrict__ L, int64_t n, double *part) {
  double v[3] = {0.0, 0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
    const float2 r = R[i], p = P[i], l = L[i];
    v[0] += (double)(r.x * r.x + r.y * r.y);
    // conj(p) * l in float
    v[1] += (double)(p.x * l.x + p.y * l.y);
    v[2] += (double)(p.x * l.y - p.y * l.x);
  }
  block_sum<3>(v);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x + 0] = v[0];
    part[3 * blockIdx.x + 1] = v[1];
    part[3 * blockIdx.x + 2] = v[2];
  }
}

// alpha = (R'R) / (P'LHS) as complex<double>, stored as complex<float>
__global__ void k_cg_alpha(const double *__restrict__ part, int nblk, Scalars *sc) {
  double v[3] = {0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblk; b += RT) {
    v[0] += part[3 * b];
    v[1] += part[3 * b + 1];
    v[2] += part[3 * b + 2];
  }
  block_sum<3>(v);
  if (threadIdx.x == 0) {
    const double rr = v[0], a = v[1], b = v[2];
    const double den = a * a + b * b;
    // (rr + 0i) / (a + bi)
    const double ar = rr * a / den, ai = -rr * b / den;
    sc->rr = rr;
    sc->pl[0] = a;
    sc->pl[1] = b;
    sc->alpha[0] = (float)ar;
    sc->alpha[1] = (float)ai;
  }
}

__global__ void __launch_bounds__(RT) k_cg_update(float2 *__restrict__ X, float2 *__restrict__ R,
                                                 const float2 *__restrict__ P, const float2 *__restrict__ L, int64_t n,
                                                 const Scalars *__restrict__ sc, double *part) {
  const float ar = sc->alpha[0], ai = sc->alpha[1];
  double v[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
    const float2 p = P[i], l = L[i];
    float2 x = X[i], r = R[i];
    x.x += ar * p.x - ai * p.y;
    x.y += ar * p.y + ai * p.x;
    r.x -= ar * l.x - ai * l.y;
    r.y -= ar * l.y + ai * l.x;
    X[i] = x;
    R[i] = r;
    v[0] += (double)(r.x * r.x + r.y * r.y);
  }
  block_sum<1>(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// beta = R'R(new) / R'R(old); residual history; iteration counter
__global__ void k_cg_beta(const double *__restrict__ part, int nblk, Scalars *sc, double *resid) {
  double v[1] = {0.0};
  for (int b = threadIdx.x; b < nblk; b += RT) v[0] += part[b];
  block_sum<1>(v);
  if (threadIdx.x == 0) {
    const double rn = v[0];
    const double bt = rn / sc->rr;
    sc->rn = rn;
    sc->beta[0] = (float)bt;
    sc->beta[1] = 0.0f;
    if (resid) resid[sc->it] = rn;
    sc->it += 1;
  }
}

__global__ void __launch_bounds__(RT) k_cg_pupdate(float2 *__restrict__ P, const float2 *__restrict__ R, int64_t n,
                                                  const Scalars *__restrict__ sc) {
  const float br = sc->beta[0], bi = sc->beta[1];
  for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
    const float2 p = P[i], r = R[i];
    P[i] = make_float2(r.x + (br * p.x - bi * p.y), r.y + (br * p.y + bi * p.x));
  }
}

mrg_status cg_dots(const float2 *R, const float2 *P, const float2 *L, int64_t n, double *part, int nblk, Scalars *sc,
                   cudaStream_t st) {
  k_cg_dots<<<nblk, RT, 0, st>>>(R, P, L, n, part);
  MRG_LAUNCHED();
  k_cg_alpha<<<1, RT, 0, st>>>(part, nblk, sc);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status cg_update(float2 *X, float2 *R, const float2 *P, const float2 *L, int64_t n, double *part, int nblk,
                     Scalars *sc, double *resid, cudaStream_t st) {
  k_cg_update<<<nblk, RT, 0, st>>>(X, R, P, L, n, sc, part);
  MRG_LAUNCHED();
  k_cg_beta<<<1, RT, 0, st>>>(part, nblk, sc, resid);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status cg_pupdate(float2 *P, const float2 *R, int64_t n, const Scalars *sc, cudaStream_t st) {
  k_cg_pupdate<<<reduce_blocks(n), RT, 0, st>>>(P, R, n, sc);
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// generic helpers
// ---------------------------------------------------------------------------
__global__ void k_interleave(const float2 *__restrict__ src, int64_t stride, int C, int64_t n, float2 *__restrict__ dst) {
  const int64_t tot = n * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = e / C;
    const int c = (int)(e - v * C);
    dst[e] = src[(int64_t)c * stride + v];
  }
}

// dst[c * stride + v] = src[v * C + c]  (plan layout back to per-coil volumes)
__global__ void k_deinterleave(const float2 *__restrict__ src, int C, int64_t n, float2 *__restrict__ dst,
                               int64_t stride) {
  const int64_t tot = n * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / n);
    const int64_t v = e - (int64_t)c * n;
    dst[(int64_t)c * stride + v] = src[v * C + c];
  }
}

mrg_status launch_deinterleave(const float2 *src, int C, int64_t n, float2 *dst, int64_t stride, cudaStream_t st) {
  k_deinterleave<<<reduce_blocks(n * C), RT, 0, st>>>(src, C, n, dst, stride);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status launch_interleave(const float2 *src, int64_t stride, int C, int64_t n, float2 *dst, cudaStream_t st) {
  k_interleave<<<reduce_blocks(n * C), RT, 0, st>>>(src, stride, C, n, dst);
  MRG_LAUNCHED();
  return MRG_OK;
}

__global__ void k_zero(uint4 *p, int64_t n16, uint8_t *tail, int ntail) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = make_uint4(0, 0, 0, 0);
  if (blockIdx.x == 0 && (int)threadIdx.x < ntail) tail[threadIdx.x] = 0;
}

__global__ void k_copy16(uint4 *__restrict__ dst, const uint4 *__restrict__ src, int64_t n16, uint8_t *dtail,
                         const uint8_t *stail, int ntail) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
  if (blockIdx.x == 0 && (int)threadIdx.x < ntail) dtail[threadIdx.x] = stail[threadIdx.x];
}

// Copy from pinned host memory (src: its device-side address) by the SMs: many loads in
// flight over the CPU-GPU link instead of one copy-engine transfer.  Both ends 16-byte aligned.
mrg_status launch_copy_from_host(void *dst, const void *src, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return MRG_OK;
  const int64_t n16 = (int64_t)(bytes / 16);
  const int ntail = (int)(bytes - n16 * 16);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n16 + 511) / 512, 8 * (int64_t)device_sms()));
  k_copy16<<<blocks, 512, 0, st>>>((uint4 *)dst, (const uint4 *)src, n16, (uint8_t *)dst + n16 * 16,
                                   (const uint8_t *)src + n16 * 16, ntail);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status launch_zero(void *p, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return MRG_OK;
  if (((uintptr_t)p & 15) != 0) {
    MRG_CUDA(cudaMemsetAsync(p, 0, bytes, st));
    return MRG_OK;
  }
  const int64_t n16 = (int64_t)(bytes / 16);
  const int ntail = (int)(bytes - n16 * 16);
  k_zero<<<reduce_blocks(n16 > 0 ? n16 : 1), RT, 0, st>>>((uint4 *)p, n16, (uint8_t *)p + n16 * 16, ntail);
  MRG_LAUNCHED();
  return MRG_OK;
}

__global__ void k_copy(float2 *__restrict__ d, const float2 *__restrict__ s, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = s[i];
}

mrg_status launch_copy(float2 *dst, const float2 *src, int64_t n, cudaStream_t st) {
  k_copy<<<reduce_blocks(n), RT, 0, st>>>(dst, src, n);
  MRG_LAUNCHED();
  return MRG_OK;
}

__global__ void k_fill(float2 *X, int64_t n, float2 v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    X[i] = v;
}

mrg_status launch_fill(float2 *X, int64_t n, float2 v, cudaStream_t st) {
  k_fill<<<reduce_blocks(n), RT, 0, st>>>(X, n, v);
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// FISTA
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_energy(const float2 *__restrict__ R, int64_t n, double *part) {
  double v[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
    const float2 r = R[i];
    v[0] += (double)(r.x * r.x + r.y * r.y);
  }
  block_sum<1>(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void k_energy_final(const double *__restrict__ part, int nblk, double *out) {
  double v[1] = {0.0};
  for (int b = threadIdx.x; b < nblk; b += RT) v[0] += part[b];
  block_sum<1>(v);
  if (threadIdx.x == 0) *out = v[0];
}

mrg_status energy(const float2 *R, int64_t n, double *part, int nblk, double *out, cudaStream_t st) {
  k_energy<<<nblk, RT, 0, st>>>(R, n, part);
  MRG_LAUNCHED();
  k_energy_final<<<1, RT, 0, st>>>(part, nblk, out);
  MRG_LAUNCHED();
  return MRG_OK;
}

// Power iteration step: X = (1/sqrt(e)) * R with e = sc->e (src/recon_lib.cpp:1894-1906).
__global__ void k_power_scale(float2 *__restrict__ X, const float2 *__restrict__ R, int64_t n, Scalars *sc) {
  const double max_eig = sqrt(sc->e);
  const float s = (float)(1. / max_eig);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 r = R[i];
    // complex<float>(s, 0) * r
    X[i] = make_float2(s * r.x - 0.0f * r.y, s * r.y + 0.0f * r.x);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->step = s;
}

mrg_status power_scale(float2 *X, const float2 *R, int64_t n, Scalars *sc, cudaStream_t st) {
  k_power_scale<<<reduce_blocks(n), RT, 0, st>>>(X, R, n, sc);
  MRG_LAUNCHED();
  return MRG_OK;
}

// fista_update (src/recon_lib.cpp:2177-2212): X = A*X + B*X_old, X_old = X.
__global__ void k_fista_momentum(float2 *__restrict__ X, float2 *__restrict__ Xo, int64_t n,
                                 const Scalars *__restrict__ sc) {
  const int it = sc->it;
  const float A = (float)(1.0 + (it - 1.0) / (it + 1.0));
  const float B = (float)(-(it - 1.0) / (it + 1.0));
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 x0 = Xo[i], x1 = X[i];
    X[i] = make_float2(A * x1.x + B * x0.x, A * x1.y + B * x0.y);
    Xo[i] = x1;
  }
}

mrg_status fista_momentum(float2 *X, float2 *Xo, int64_t n, const Scalars *sc, int fista, cudaStream_t st) {
  if (!fista) return MRG_OK;
  k_fista_momentum<<<reduce_blocks(n), RT, 0, st>>>(X, Xo, n, sc);
  MRG_LAUNCHED();
  return MRG_OK;
}

// R'R (FP64) then X -= step * R  (src/recon_lib.cpp:2072-2105)
__global__ void __launch_bounds__(RT) k_grad_step(float2 *__restrict__ X, const float2 *__restrict__ R, int64_t n,
                                                 const Scalars *__restrict__ sc, double *part) {
  const float s = sc->step;
  double v[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
    const float2 r = R[i];
    v[0] += (double)(r.x * r.x + r.y * r.y);
    float2 x = X[i];
    // R *= complex<float>(step, 0); X -= R
    x.x -= (r.x * s - r.y * 0.0f);
    x.y -= (r.x * 0.0f + r.y * s);
    X[i] = x;
  }
  block_sum<1>(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void k_grad_final(const double *__restrict__ part, int nblk, Scalars *sc, double *resid) {
  double v[1] = {0.0};
  for (int b = threadIdx.x; b < nblk; b += RT) v[0] += part[b];
  block_sum<1>(v);
  if (threadIdx.x == 0) {
    sc->e = v[0];
    if (resid) resid[sc->it] = v[0];
  }
}

mrg_status grad_step(float2 *X, const float2 *R, int64_t n, const Scalars *sc, double *part, int nblk, double *resid,
                     cudaStream_t st) {
  k_grad_step<<<nblk, RT, 0, st>>>(X, R, n, sc, part);
  MRG_LAUNCHED();
  k_grad_final<<<1, RT, 0, st>>>(part, nblk, const_cast<Scalars *>(sc), resid);
  MRG_LAUNCHED();
  return MRG_OK;
}

__global__ void k_bump(Scalars *sc) { sc->it += 1; }

mrg_status bump_iteration(Scalars *sc, cudaStream_t st) {
  k_bump<<<1, 1, 0, st>>>(sc);
  MRG_LAUNCHED();
  return MRG_OK;
}

}  // namespace mrg
