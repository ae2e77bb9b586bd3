// Locally low rank in time (LOWRANKCOIL::update_threshold / thresh with
// dim = 0, Ne = 1; src/clear.cpp:233-556).
//
// A block is the Np x Nt matrix A (Np = bx*by*bz voxels, Nt frames) gathered
// with periodic wrap at a circular shift.  One CTA per block forms the Gram
// matrix G = A^H A in FP64, diagonalises it with a cyclic Hermitian Jacobi
// sweep run by one warp (G = V diag(s^2) V^H), and
//   update_threshold: s1 = sqrt(lambda_max) per block, then the median of the
//                     non-zero s1 times (1 + clear_amp*exp(-iter/clear_t2));
//   thresh:           A <- A V diag(max(s - tau, 0)/s) V^H, which equals
//                     U diag(max(s - tau, 0)) V^H of the reference's SVD.
// Block shifts come from a device table so the pass can be graph-captured.
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

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }

__global__ void __launch_bounds__(256) k_llr(const LlrArgs a) {
  extern __shared__ float2 A[];  // [Np][Nt]
  __shared__ double2 G[LLR_MAXT][LLR_MAXT], V[LLR_MAXT][LLR_MAXT], Mx[LLR_MAXT][LLR_MAXT];
  __shared__ double lam[LLR_MAXT];
  const int Nt = a.Nt;
  const int bx = a.bs[0], by = a.bs[1], bz = a.bs[2];
  const int Np = bx * by * bz;
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
  // gather (periodic wrap, clear.cpp:436-448)
  for (int e = threadIdx.x; e < Np * Nt; e += blockDim.x) {
    const int v = e % Np, t = e / Np;
    const int ii = v % bx, jj = (v / bx) % by, kk = v / (bx * by);
    const int px = (i0 + ii + a.N[0]) % a.N[0], py = (j0 + jj + a.N[1]) % a.N[1], pz = (k0 + kk + a.N[2]) % a.N[2];
    A[v * Nt + t] = a.X[t * a.vstride + ((int64_t)pz * a.N[1] + py) * a.N[0] + px];
  }
  __syncthreads();
  // Gram matrix in FP64 (upper triangle, mirrored)
  for (int e = threadIdx.x; e < Nt * Nt; e += blockDim.x) {
    const int p = e / Nt, q = e % Nt;
    if (p > q) continue;
    double re = 0.0, im = 0.0;
    for (int v = 0; v < Np; v++) {
      const float2 x = A[v * Nt + p], y = A[v * Nt + q];
      re += (double)x.x * y.x + (double)x.y * y.y;
      im += (double)x.x * y.y - (double)x.y * y.x;
    }
    G[p][q] = make_double2(re, im);
    G[q][p] = make_double2(re, -im);
  }
  for (int e = threadIdx.x; e < Nt * Nt; e += blockDim.x) V[e / Nt][e % Nt] = make_double2((e / Nt) == (e % Nt), 0.0);
  __syncthreads();
  // cyclic Hermitian Jacobi, warp 0 (lane k updates element k of the two rows / columns)
  if (threadIdx.x < 32) {
    const int k = threadIdx.x;
    for (int sweep = 0; sweep < 40; sweep++) {
      double off = 0.0, diag = 0.0;
      for (int p = 0; p < Nt; p++) {
        diag += G[p][p].x * G[p][p].x;
        for (int q = p + 1; q < Nt; q++) off += G[p][q].x * G[p][q].x + G[p][q].y * G[p][q].y;
      }
      if (off <= 1e-30 * diag || off == 0.0) break;
      for (int p = 0; p < Nt - 1; p++) {
        for (int q = p + 1; q < Nt; q++) {
          const double2 gpq = G[p][q];
          const double r = sqrt(gpq.x * gpq.x + gpq.y * gpq.y);
          __syncwarp();
          if (r <= 1e-300) continue;
          const double2 e = make_double2(gpq.x / r, gpq.y / r);  // e^{i phi}
          const double tau = (G[q][q].x - G[p][p].x) / (2.0 * r);
          const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
          const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
          const double2 se = make_double2(s * e.x, s * e.y);          // s e^{i phi}
          const double2 sec = make_double2(s * e.x, -s * e.y);        // s e^{-i phi}
          __syncwarp();
          // G <- G J: col p = c G[:,p] - s e^{-i phi} G[:,q]; col q = s e^{i phi} G[:,p] + c G[:,q]
          if (k < Nt) {
            const double2 gp = G[k][p], gq = G[k][q];
            const double2 a1 = zmul(sec, gq), a2 = zmul(se, gp);
            G[k][p] = make_double2(c * gp.x - a1.x, c * gp.y - a1.y);
            G[k][q] = make_double2(a2.x + c * gq.x, a2.y + c * gq.y);
            const double2 vp = V[k][p], vq = V[k][q];
            const double2 b1 = zmul(sec, vq), b2 = zmul(se, vp);
            V[k][p] = make_double2(c * vp.x - b1.x, c * vp.y - b1.y);
            V[k][q] = make_double2(b2.x + c * vq.x, b2.y + c * vq.y);
          }
          __syncwarp();
          // G <- J^H G: row p = c G[p,:] - s e^{i phi} G[q,:]; row q = s e^{-i phi} G[p,:] + c G[q,:]
          if (k < Nt) {
            const double2 hp = G[p][k], hq = G[q][k];
            const double2 a1 = zmul(se, hq), a2 = zmul(sec, hp);
            G[p][k] = make_double2(c * hp.x - a1.x, c * hp.y - a1.y);
            G[q][k] = make_double2(a2.x + c * hq.x, a2.y + c * hq.y);
          }
          __syncwarp();
          if (k == 0) {
            G[p][q] = make_double2(0.0, 0.0);
            G[q][p] = make_double2(0.0, 0.0);
            G[p][p].y = 0.0;
            G[q][q].y = 0.0;
          }
          __syncwarp();
        }
      }
    }
    if (k < Nt) lam[k] = fmax(G[k][k].x, 0.0);
  }
  __syncthreads();
  if (a.mode == 0) {
    if (threadIdx.x == 0) {
      double m = 0.0;
      for (int j = 0; j < Nt; j++) m = fmax(m, lam[j]);
      a.sig[b] = sqrt(m);
    }
    return;
  }
  // M = V diag(f) V^H with f = max(s - tau, 0) / s
  const double tau = a.alpha * (double)(*a.smax) / a.block_iter;  // clear.cpp:397, :497-499
  for (int e = threadIdx.x; e < Nt * Nt; e += blockDim.x) {
    const int r = e / Nt, cidx = e % Nt;
    double2 acc = make_double2(0.0, 0.0);
    for (int j = 0; j < Nt; j++) {
      const double s = sqrt(lam[j]);
      const double f = (s > 0.0) ? fmax(s - tau, 0.0) / s : 0.0;
      const double2 t = zmul(V[r][j], zconj(V[cidx][j]));
      acc.x += f * t.x;
      acc.y += f * t.y;
    }
    Mx[r][cidx] = acc;
  }
  __syncthreads();
  // A' = A M, scatter back
  for (int e = threadIdx.x; e < Np * Nt; e += blockDim.x) {
    const int v = e % Np, t = e / Np;
    double2 acc = make_double2(0.0, 0.0);
    for (int j = 0; j < Nt; j++) {
      const float2 x = A[v * Nt + j];
      const double2 m = Mx[j][t];
      acc.x += (double)x.x * m.x - (double)x.y * m.y;
      acc.y += (double)x.x * m.y + (double)x.y * m.x;
    }
    const int ii = v % bx, jj = (v / bx) % by, kk = v / (bx * by);
    const int px = (i0 + ii + a.N[0]) % a.N[0], py = (j0 + jj + a.N[1]) % a.N[1], pz = (k0 + kk + a.N[2]) % a.N[2];
    a.X[t * a.vstride + ((int64_t)pz * a.N[1] + py) * a.N[0] + px] = make_float2((float)acc.x, (float)acc.y);
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
  const size_t smem = sizeof(float2) * (size_t)Np * a.Nt;
  if (a.Nt > LLR_MAXT || a.Nt < 1) {
    set_error("low-rank blocks support 1.." + std::to_string(LLR_MAXT) + " frames");
    return MRG_ERR_UNSUPPORTED;
  }
  if (smem > 200 * 1024) {
    set_error("low-rank block too large");
    return MRG_ERR_UNSUPPORTED;
  }
  static bool attr = false;
  if (!attr) {
    MRG_CUDA(cudaFuncSetAttribute(k_llr, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  k_llr<<<nblocks, 256, smem, st>>>(a);
  MRG_LAUNCHED();
  return MRG_OK;
}

static void llr_geom(LlrArgs &a, float2 *X, int Nt, const int N[3], const int bs[3], int &nblocks) {
  a.X = X;
  a.vstride = (int64_t)N[0] * N[1] * N[2];
  a.Nt = Nt;
  nblocks = 1;
  for (int d = 0; d < 3; d++) {
    a.N[d] = N[d];
    a.bs[d] = std::min(bs[d], N[d]);
    a.nb[d] = N[d] / a.bs[d];
    nblocks *= a.nb[d];
  }
}

int llr_block_count(const int N[3], const int bs[3]) {
  int nb = 1;
  for (int d = 0; d < 3; d++) nb *= N[d] / std::min(bs[d], N[d]);
  return nb;
}

mrg_status llr_update_into(const float2 *X, int Nt, const int N[3], const int bs[3], float amp, float t2,
                           const Scalars *sc, int iter_fixed, double *sig, double *work, float *smax, cudaStream_t st) {
  LlrArgs a;
  memset(&a, 0, sizeof(a));
  int nblocks;
  llr_geom(a, const_cast<float2 *>(X), Nt, N, bs, nblocks);
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
  const int nblocks = llr_block_count(N, bs);
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
  int nblocks;
  llr_geom(a, X, Nt, N, bs, nblocks);
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
