// Locally low rank in time (LOWRANKCOIL::update_threshold / thresh with
// dim = 0, Ne = 1; src/clear.cpp:233-556).
//
// A block is the Np x Nt matrix A (Np = bx*by*bz voxels, Nt frames) gathered
// with periodic wrap at a circular shift.  One CTA per block takes its SVD by a
// one-sided Jacobi in FP32 in shared memory (jacobi.cuh; the reference uses
// Armadillo's double-precision svd_econ, and FP64 arithmetic is slow on this part:
// the earlier FP64 Gram + Hermitian Jacobi kernel took 16 ms per pass at 128^3 x 10
// frames in 8^3 blocks), and
//   update_threshold: s1 = the largest singular value per block, then the median of
//                     the non-zero s1 times (1 + clear_amp*exp(-iter/clear_t2));
//   thresh:           A <- U diag(max(s - tau, 0)) V^H.
// Block shifts come from a device table so the pass can be graph-captured.
#include "jacobi.cuh"
#include "mrg_internal.h"

namespace mrg {

constexpr int LLR_MAXT = 16;  // frames per block handled by this build

struct LlrArgs {
  float2 *X;
  int64_t vstride;
  int Nt;
  int N[3], bs[3], nb[3];
  const int *shifts;  // [.. ][3]; NULL = no shift
  const Scalars *sc;
  int per_it, off;
  int mode;           // 0: sigma_1 -> sig; 1: threshold with tau
  double *sig;
  const float *smax;  // device smax (mode 1)
  double alpha;       // clear_alpha_time (mode 1); tau = alpha * smax / block_iter
  int block_iter;
};

// One CTA per block: gather A (Np x Nt, periodic wrap), one-sided Jacobi in FP32
// (jacobi.cuh): A W has orthogonal columns whose norms are the singular values s_j and W
// holds the right singular vectors, so
//   mode 0: sig[b] = max_j s_j (sigma_1 of the block);
//   mode 1: A <- (A W) diag(f) W^H, f_j = max(s_j - tau, 0) / s_j  (= U diag(max(s - tau, 0)) V^H).
__global__ void __launch_bounds__(256) k_llr(const LlrArgs a) {
  extern __shared__ __align__(16) float2 A[];  // [Np][ld], then W [Nt][JAC_LDV], then s [Nt]
  __shared__ unsigned s_off;
  __shared__ float s_fl;
  const int Nt = a.Nt, ld = Nt | 1;  // odd row pitch: a warp's column reads spread over the banks
  const int bx = a.bs[0], by = a.bs[1], bz = a.bs[2];
  const int Np = bx * by * bz;
  float2 *W = A + (size_t)Np * ld;
  float *sg = reinterpret_cast<float *>(W + (size_t)Nt * JAC_LDV);
  const int b = blockIdx.x;
  // block order as clear.cpp:249-264 (i outer, k inner) -- any order gives the same result
  const int bk = b % a.nb[2], bj = (b / a.nb[2]) % a.nb[1], bi = b / (a.nb[1] * a.nb[2]);
  int sh[3] = {0, 0, 0};
  if (a.shifts) {
    const int base = (a.sc ? a.sc->it : 0) * a.per_it + a.off;
    sh[0] = a.shifts[base + 0];
    sh[1] = a.shifts[base + 1];
    sh[2] = a.shifts[base + 2];
  }
  const int i0 = bi * bx + sh[0], j0 = bj * by + sh[1], k0 = bk * bz + sh[2];
  auto voxel = [&](int v) -> int64_t {  // periodic wrap (clear.cpp:436-448)
    const int ii = v % bx, jj = (v / bx) % by, kk = v / (bx * by);
    const int px = (i0 + ii + a.N[0]) % a.N[0], py = (j0 + jj + a.N[1]) % a.N[1], pz = (k0 + kk + a.N[2]) % a.N[2];
    return ((int64_t)pz * a.N[1] + py) * a.N[0] + px;
  };
  // gather: consecutive threads read consecutive voxels of one frame
  for (int e = threadIdx.x; e < Np * Nt; e += blockDim.x) {
    const int v = e % Np, t = e / Np;
    A[v * ld + t] = a.X[t * a.vstride + voxel(v)];
  }
  __syncthreads();
  jacobi_onesided_f32(A, Np, Nt, ld, W, sg, &s_off, &s_fl);
  if (a.mode == 0) {
    if (threadIdx.x == 0) {
      float m = 0.f;
      for (int j = 0; j < Nt; j++) m = fmaxf(m, sg[j]);
      a.sig[b] = (double)m;
    }
    return;
  }
  const double tau = a.alpha * (double)(*a.smax) / a.block_iter;  // clear.cpp:397, :497-499
  __syncthreads();
  if (threadIdx.x < Nt) {
    const float sj = sg[threadIdx.x];
    sg[threadIdx.x] = sj > 0.f ? (float)(fmax((double)sj - tau, 0.0) / (double)sj) : 0.f;
  }
  __syncthreads();
  // A' = (A W) diag(f) W^H, scattered back (clear.cpp:530-551)
  for (int e = threadIdx.x; e < Np * Nt; e += blockDim.x) {
    const int v = e % Np, t = e / Np;
    float2 acc = make_float2(0.f, 0.f);
    for (int j = 0; j < Nt; j++) {
      const float2 x = A[v * ld + j], w = W[t * JAC_LDV + j];
      const float f = sg[j];
      acc.x += f * (x.x * w.x + x.y * w.y);  // x f conj(w)
      acc.y += f * (x.y * w.x - x.x * w.y);
    }
    a.X[t * a.vstride + voxel(v)] = acc;
  }
}

// Median of the non-zero sigma_1 (bitonic sort of a padded copy in one CTA),
// times the amplitude schedule (clear.cpp:343-347).
__global__ void k_llr_median(const double *__restrict__ sig, int n, double *work, int npow2, float amp, float t2,
                             const Scalars *sc, int iter_fixed, float *smax) {
  for (int i = threadIdx.x; i < npow2; i += blockDim.x) work[i] = (i < n) ? sig[i] : __longlong_as_double(0x7ff0000000000000LL);
  __syncthreads();
  for (int k = 2; k <= npow2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const double a = work[i], b = work[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            work[i] = b;
            work[l] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    int z = 0;
    while (z < n && work[z] == 0.0) z++;
    const int m = n - z;
    double med = 0.0;
    if (m > 0) med = (m & 1) ? work[z + m / 2] : 0.5 * (work[z + m / 2 - 1] + work[z + m / 2]);
    const int iter = sc ? sc->it : iter_fixed;
    const float ampv = 1 + amp * expf(-((float)iter) / t2);
    *smax = (float)(med * ampv);
  }
}

mrg_status llr_median(const double *sig, int n, double *work, float amp, float t2, int iter, float *smax,
                      cudaStream_t st) {
  int np2 = 1;
  while (np2 < n) np2 <<= 1;
  k_llr_median<<<1, 1024, 0, st>>>(sig, n, work, np2, amp, t2, nullptr, iter, smax);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status llr_alloc(LlrWork &w, int nblocks) {
  if (w.nb >= nblocks && w.sig) return MRG_OK;
  llr_free(w);
  int np2 = 1;
  while (np2 < nblocks) np2 <<= 1;
  MRG_CUDA(cudaMalloc(&w.sig, sizeof(double) * (size_t)(nblocks + np2)));
  MRG_CUDA(cudaMalloc(&w.smax, sizeof(float)));
  w.nb = nblocks;
  return MRG_OK;
}

void llr_free(LlrWork &w) {
  cudaFree(w.sig);
  cudaFree(w.smax);
  w.sig = nullptr;
  w.smax = nullptr;
  w.nb = 0;
}

static mrg_status llr_launch(const LlrArgs &a, int nblocks, cudaStream_t st) {
  const int Np = a.bs[0] * a.bs[1] * a.bs[2];
  const size_t smem = sizeof(float2) * ((size_t)Np * (a.Nt | 1) + (size_t)a.Nt * JAC_LDV) + sizeof(float) * 16;
  if (a.Nt > LLR_MAXT || a.Nt < 1) {
    set_error("low-rank blocks support 1.." + std::to_string(LLR_MAXT) + " frames");
    return MRG_ERR_UNSUPPORTED;
  }
  if (smem > 200 * 1024) {
    set_error("low-rank block too large");
    return MRG_ERR_UNSUPPORTED;
  }
  static DeviceOnce once;
  MRG_TRY(device_once(once, []() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_llr, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    return MRG_OK;
  }));
  k_llr<<<nblocks, 256, smem, st>>>(a);
  MRG_LAUNCHED();
  return MRG_OK;
}

// Block geometry of one launch; the block count must fit a grid dimension and the int
// indices of the median's sort.
static mrg_status llr_geom(LlrArgs &a, float2 *X, int Nt, const int N[3], const int bs[3], int &nblocks) {
  a.X = X;
  a.vstride = (int64_t)N[0] * N[1] * N[2];
  a.Nt = Nt;
  int64_t nb = 1;
  for (int d = 0; d < 3; d++) {
    if (bs[d] < 1 || N[d] < 1) {
      set_error("low-rank block and image sizes must be positive");
      return MRG_ERR_INVALID;
    }
    a.N[d] = N[d];
    a.bs[d] = std::min(bs[d], N[d]);
    a.nb[d] = N[d] / a.bs[d];
    nb *= a.nb[d];
  }
  if (nb > (int64_t)(1 << 30)) {
    set_error("too many low-rank blocks (" + std::to_string(nb) + ") for one launch");
    return MRG_ERR_UNSUPPORTED;
  }
  nblocks = (int)nb;
  return MRG_OK;
}

int64_t llr_block_count(const int N[3], const int bs[3]) {
  int64_t nb = 1;
  for (int d = 0; d < 3; d++) nb *= N[d] / std::min(bs[d], N[d]);
  return nb;
}

mrg_status llr_update_into(const float2 *X, int Nt, const int N[3], const int bs[3], float amp, float t2,
                           const Scalars *sc, int iter_fixed, double *sig, double *work, float *smax, cudaStream_t st) {
  LlrArgs a;
  memset(&a, 0, sizeof(a));
  int nblocks = 0;
  MRG_TRY(llr_geom(a, const_cast<float2 *>(X), Nt, N, bs, nblocks));
  a.mode = 0;
  a.sig = sig;
  MRG_TRY(llr_launch(a, nblocks, st));
  int np2 = 1;
  while (np2 < nblocks) np2 <<= 1;
  k_llr_median<<<1, 1024, 0, st>>>(sig, nblocks, work, np2, amp, t2, sc, iter_fixed, smax);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status llr_update_ex(const float2 *X, int Nt, const int N[3], const int bs[3], float amp, float t2,
                         const Scalars *sc, int iter_fixed, LlrWork &w, cudaStream_t st) {
  const int64_t nb = llr_block_count(N, bs);
  if (nb > (int64_t)(1 << 30)) {
    set_error("too many low-rank blocks (" + std::to_string(nb) + ") for one launch");
    return MRG_ERR_UNSUPPORTED;
  }
  const int nblocks = (int)nb;
  MRG_TRY(llr_alloc(w, nblocks));
  return llr_update_into(X, Nt, N, bs, amp, t2, sc, iter_fixed, w.sig, w.sig + nblocks, w.smax, st);
}

mrg_status llr_update(const float2 *X, int Nt, const int N[3], const int bs[3], float amp, float t2,
                      const int *iter_dev, LlrWork &w, cudaStream_t st) {
  (void)iter_dev;
  return llr_update_ex(X, Nt, N, bs, amp, t2, nullptr, 0, w, st);
}

mrg_status llr_apply_ex(float2 *X, int Nt, const int N[3], const int bs[3], int block_iter, float alpha,
                        const int *shifts, const Scalars *sc, int per_it, int off_base, const float *smax_dev,
                        cudaStream_t st) {
  if (alpha == 0.0f) return MRG_OK;
  LlrArgs a;
  memset(&a, 0, sizeof(a));
  int nblocks = 0;
  MRG_TRY(llr_geom(a, X, Nt, N, bs, nblocks));
  a.mode = 1;
  a.smax = smax_dev;
  a.alpha = (double)alpha;
  a.block_iter = block_iter;
  a.sc = sc;
  a.per_it = per_it;
  for (int it = 0; it < block_iter; it++) {
    a.shifts = shifts;
    a.off = off_base + 3 * it;
    MRG_TRY(llr_launch(a, nblocks, st));
  }
  return MRG_OK;
}

mrg_status llr_apply(float2 *X, int Nt, const int N[3], const int bs[3], int block_iter, float alpha,
                     const int *shifts_dev, const float *smax_dev, cudaStream_t st) {
  return llr_apply_ex(X, Nt, N, bs, block_iter, alpha, shifts_dev, nullptr, 0, 0, smax_dev, st);
}

}  // namespace mrg
