// CLEAR: coil low rank (LOWRANKCOIL with dim = 2, src/clear.cpp:99-232, :561-813,
// :815-914) on per-coil image stacks stored [frame][voxel][coil] (coil innermost, the
// layout the operators read maps in), and the vector steps of the CLEAR gradient loop
// (src/recon_lib.cpp:1025-1238).
//
// A block is the matrix A of R = frames * bx*by*bz rows (frames stacked, as the
// reference's gather counts over encodes, frames and voxels) and C columns (coils),
// gathered with periodic wrap at a circular shift.  One CTA per block forms the Gram
// matrix G = A^H A in FP64, diagonalises it with a cyclic Hermitian Jacobi sweep run by
// one warp (lane k owns row / column k, C <= 32), and
//   thresh:  A <- A V diag(max(s - tau, 0)/s) V^H  (= U diag(max(s - tau, 0)) V^H),
//            tau = clear_alpha_coil * smax / block_iter (src/clear.cpp:589-598, :715);
//   combine: image = A v1, v1 the right singular vector of the largest singular value
//            (src/clear.cpp:887-890).  A singular vector is defined up to a unit phase;
//            v1 is scaled so that its largest-magnitude component is real and positive.
// update_threshold with dim = 2 gathers every coil into column t (src/clear.cpp:185-199:
// A(count, t) inside the coil loop, count restarting per coil), so the last coil's block
// is what remains and sigma_1 = max over frames of its block norm; that is what is
// computed here, then the median of the non-zero sigma_1 times (1 + amp exp(-iter/t2)).
#include "jacobi.cuh"
#include "mrg_internal.h"

namespace mrg {

namespace {

constexpr int CL_MAXC = 32;  // coils per block matrix handled by this build
constexpr int CL_LD = CL_MAXC;

struct CoilLlrArgs {
  float2 *X;          // [T][nvox][C]
  float2 *out;        // combine: [T][nvox]
  int T, C;
  int N[3], bs[3], nb[3];
  int64_t nvox;
  const int *shift;   // 3 ints (device) or NULL
  int mode;           // 0: sigma_1 of the last coil; 1: threshold; 2: combine
  double *sig;
  const float *smax;
  double alpha;
  int block_iter;
};

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }

// Cyclic Hermitian Jacobi on G (n x n, leading dimension CL_LD), accumulating the
// eigenvectors in V; warp-wide (lane k updates element k).  lam = the eigenvalues.  FP64
// division and square root are slow on this part, so lane 0 alone computes each rotation
// and shuffles it to the warp, and the off-diagonal norm is summed lane-strided.
__device__ void herm_jacobi(double2 *G, double2 *V, double *lam, int n) {
  const int k = threadIdx.x & 31;
  for (int sweep = 0; sweep < 40; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int e = k; e < n * n; e += 32) {
      const int p = e / n, q = e - p * n;
      const double2 g = G[p * CL_LD + q];
      if (q > p) off += g.x * g.x + g.y * g.y;
      else if (q == p) diag += g.x * g.x;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      diag += __shfl_xor_sync(0xffffffffu, diag, o);
    }
    if (off <= 1e-26 * diag || off == 0.0) break;  // |offdiag| <= 1e-13 |diag|
    for (int p = 0; p < n - 1; p++) {
      for (int q = p + 1; q < n; q++) {
        double c = 1.0, sx = 0.0, sy = 0.0;  // rotation: c and s e^{i phi}
        int skip = 0;
        if (k == 0) {
          const double2 gpq = G[p * CL_LD + q];
          const double r = sqrt(gpq.x * gpq.x + gpq.y * gpq.y);
          if (r <= 1e-300) {
            skip = 1;
          } else {
            const double tau = (G[q * CL_LD + q].x - G[p * CL_LD + p].x) / (2.0 * r);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            const double sr = t * c / r;  // s / r: s e^{i phi} = (s / r) g_pq
            sx = sr * gpq.x;
            sy = sr * gpq.y;
          }
        }
        skip = __shfl_sync(0xffffffffu, skip, 0);
        if (skip) continue;
        c = __shfl_sync(0xffffffffu, c, 0);
        sx = __shfl_sync(0xffffffffu, sx, 0);
        sy = __shfl_sync(0xffffffffu, sy, 0);
        const double2 se = make_double2(sx, sy), sec = make_double2(sx, -sy);
        if (k < n) {  // G <- G J, V <- V J
          const double2 gp = G[k * CL_LD + p], gq = G[k * CL_LD + q];
          const double2 a1 = zmul(sec, gq), a2 = zmul(se, gp);
          G[k * CL_LD + p] = make_double2(c * gp.x - a1.x, c * gp.y - a1.y);
          G[k * CL_LD + q] = make_double2(a2.x + c * gq.x, a2.y + c * gq.y);
          const double2 vp = V[k * CL_LD + p], vq = V[k * CL_LD + q];
          const double2 b1 = zmul(sec, vq), b2 = zmul(se, vp);
          V[k * CL_LD + p] = make_double2(c * vp.x - b1.x, c * vp.y - b1.y);
          V[k * CL_LD + q] = make_double2(b2.x + c * vq.x, b2.y + c * vq.y);
        }
        __syncwarp();
        if (k < n) {  // G <- J^H G
          const double2 hp = G[p * CL_LD + k], hq = G[q * CL_LD + k];
          const double2 a1 = zmul(se, hq), a2 = zmul(sec, hp);
          G[p * CL_LD + k] = make_double2(c * hp.x - a1.x, c * hp.y - a1.y);
          G[q * CL_LD + k] = make_double2(a2.x + c * hq.x, a2.y + c * hq.y);
        }
        __syncwarp();
        if (k == 0) {
          G[p * CL_LD + q] = make_double2(0.0, 0.0);
          G[q * CL_LD + p] = make_double2(0.0, 0.0);
          G[p * CL_LD + p].y = 0.0;
          G[q * CL_LD + q].y = 0.0;
        }
        __syncwarp();
      }
    }
  }
  if (k < n) lam[k] = fmax(G[k * CL_LD + k].x, 0.0);
}

template <bool SA>
__global__ void __launch_bounds__(256) k_llr_coil(const CoilLlrArgs a) {
  extern __shared__ __align__(16) unsigned char cl_sm[];
  double2 *G = reinterpret_cast<double2 *>(cl_sm);
  double2 *V = G + CL_LD * CL_LD;
  double2 *Mx = V + CL_LD * CL_LD;
  double *lam = reinterpret_cast<double *>(Mx + CL_LD * CL_LD);
  double *red = lam + CL_LD;                          // 256 doubles
  float2 *As = reinterpret_cast<float2 *>(red + 256);  // [R][C] when SA
  __shared__ int jmax;
  __shared__ double2 ph;
  const int C = a.C, T = a.T;
  const int bx = a.bs[0], by = a.bs[1], bz = a.bs[2];
  const int Np = bx * by * bz, R = T * Np;
  const int b = blockIdx.x;
  const int bi = b % a.nb[0], bj = (b / a.nb[0]) % a.nb[1], bk = b / (a.nb[0] * a.nb[1]);
  int sh[3] = {0, 0, 0};
  if (a.shift) {
    sh[0] = a.shift[0];
    sh[1] = a.shift[1];
    sh[2] = a.shift[2];
  }
  const int i0 = bi * bx + sh[0], j0 = bj * by + sh[1], k0 = bk * bz + sh[2];
  // element offset of row r = t * Np + v (voxel v of the block, x fastest), periodic wrap
  // (src/clear.cpp:645-648)
  auto row = [&](int r) -> int64_t {
    const int t = r / Np, v = r - t * Np;
    const int ii = v % bx, jj = (v / bx) % by, kk = v / (bx * by);
    const int px = (i0 + ii + a.N[0]) % a.N[0], py = (j0 + jj + a.N[1]) % a.N[1], pz = (k0 + kk + a.N[2]) % a.N[2];
    return ((int64_t)t * a.nvox + ((int64_t)pz * a.N[1] + py) * a.N[0] + px) * C;
  };
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  if (a.mode == 0) {
    // sigma_1 = max over frames of the norm of the last coil's block
    double best = 0.0;
    for (int t = 0; t < T; t++) {
      double s = 0.0;
      for (int v = threadIdx.x; v < Np; v += blockDim.x) {
        const float2 x = a.X[row(t * Np + v) + (C - 1)];
        s += (double)x.x * x.x + (double)x.y * x.y;
      }
      red[threadIdx.x] = s;
      __syncthreads();
      for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
      }
      best = fmax(best, red[0]);
      __syncthreads();
    }
    if (threadIdx.x == 0) a.sig[b] = sqrt(best);
    return;
  }
  // gather (src/clear.cpp:681-698)
  if (SA) {
    for (int r = warp; r < R; r += nwarp)
      if (lane < C) As[r * C + lane] = a.X[row(r) + lane];
    __syncthreads();
  }
  if (SA && C <= 16) {
    // One-sided Jacobi on the columns of the block matrix in shared memory, in FP32 (FP64 is
    // slow on this part): A W = U diag(s) column by column, W = V accumulated.  Round-robin
    // rounds over the coil columns; warp w rotates pairs w, w + 8, ... of a round.  Measured
    // against the FP64 oracle: <= 2e-6 per threshold application up to 16 coils, 1.4e-5 at
    // 32 coils, so wider blocks take the FP64 Gram path below.
    float2 *Vf = reinterpret_cast<float2 *>(G);  // V[c][j] at c * JAC_LDV + j
    float *sg = reinterpret_cast<float *>(lam);  // column norms, then threshold factors
    __shared__ unsigned s_off;
    __shared__ float s_fl;
    jacobi_onesided_f32(As, R, C, C, Vf, sg, &s_off, &s_fl);
    if (a.mode == 2) {
      // combine: A v1 = column jmax of A W, times the phase that makes v1's largest
      // component real and positive
      if (threadIdx.x == 0) {
        int j = 0;
        for (int q = 1; q < C; q++)
          if (sg[q] > sg[j]) j = q;
        jmax = j;
        int m = 0;
        float mm = -1.f;
        for (int q = 0; q < C; q++) {
          const float2 x = Vf[q * JAC_LDV + j];
          const float n2 = x.x * x.x + x.y * x.y;
          if (n2 > mm) mm = n2, m = q;
        }
        const float2 x = Vf[m * JAC_LDV + j];
        const float n = sqrtf(mm);
        ph = (n > 0.f) ? make_double2(x.x / n, -x.y / n) : make_double2(1.0, 0.0);
      }
      __syncthreads();
      const float px = (float)ph.x, py = (float)ph.y;
      for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const float2 x = As[r * C + jmax];
        a.out[row(r) / C] = make_float2(x.x * px - x.y * py, x.x * py + x.y * px);
      }
      return;
    }
    // threshold: A' = (A W) diag(f) V^H, f = max(s - tau, 0) / s
    const double tau = a.alpha * (double)(*a.smax) / a.block_iter;
    __syncthreads();
    if (threadIdx.x < C) {
      const float sj = sg[threadIdx.x];
      sg[threadIdx.x] = sj > 0.f ? (float)(fmax((double)sj - tau, 0.0) / (double)sj) : 0.f;
    }
    __syncthreads();
    for (int r = warp; r < R; r += nwarp) {
      float2 acc = make_float2(0.f, 0.f);
      if (lane < C)
        for (int j = 0; j < C; j++) {
          const float2 x = As[r * C + j], v = Vf[lane * JAC_LDV + j];
          const float f = sg[j];
          acc.x += f * (x.x * v.x + x.y * v.y);  // x f conj(v)
          acc.y += f * (x.y * v.x - x.x * v.y);
        }
      if (lane < C) a.X[row(r) + lane] = acc;
    }
    return;
  }
  auto ld = [&](int r, int c) -> float2 { return SA ? As[r * C + c] : a.X[row(r) + c]; };
  // Gram matrix G = A^H A in FP64 (upper triangle, mirrored)
  for (int e = threadIdx.x; e < C * C; e += blockDim.x) {
    const int p = e / C, q = e % C;
    if (p > q) continue;
    double re = 0.0, im = 0.0;
    for (int r = 0; r < R; r++) {
      const float2 x = ld(r, p), y = ld(r, q);
      re += (double)x.x * y.x + (double)x.y * y.y;
      im += (double)x.x * y.y - (double)x.y * y.x;
    }
    G[p * CL_LD + q] = make_double2(re, im);
    G[q * CL_LD + p] = make_double2(re, -im);
  }
  for (int e = threadIdx.x; e < C * C; e += blockDim.x) V[(e / C) * CL_LD + e % C] = make_double2((e / C) == (e % C), 0.0);
  __syncthreads();
  if (warp == 0) herm_jacobi(G, V, lam, C);
  __syncthreads();
  if (a.mode == 2) {
    // combine: v1 of the largest eigenvalue, phase fixed by its largest component
    if (threadIdx.x == 0) {
      int j = 0;
      for (int q = 1; q < C; q++)
        if (lam[q] > lam[j]) j = q;
      jmax = j;
      int m = 0;
      double mm = -1.0;
      for (int q = 0; q < C; q++) {
        const double2 x = V[q * CL_LD + j];
        const double n2 = x.x * x.x + x.y * x.y;
        if (n2 > mm) mm = n2, m = q;
      }
      const double2 x = V[m * CL_LD + j];
      const double n = sqrt(mm);
      ph = (n > 0.0) ? make_double2(x.x / n, -x.y / n) : make_double2(1.0, 0.0);  // conj(x)/|x|
    }
    __syncthreads();
    const double2 vv = lane < C ? zmul(V[lane * CL_LD + jmax], ph) : make_double2(0.0, 0.0);
    for (int r = warp; r < R; r += nwarp) {
      double2 acc = make_double2(0.0, 0.0);
      if (lane < C) {
        const float2 x = ld(r, lane);
        acc.x = (double)x.x * vv.x - (double)x.y * vv.y;
        acc.y = (double)x.x * vv.y + (double)x.y * vv.x;
      }
      for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
      }
      if (lane == 0) a.out[row(r) / C] = make_float2((float)acc.x, (float)acc.y);
    }
    return;
  }
  // M = V diag(f) V^H with f = max(s - tau, 0) / s  (src/clear.cpp:712-722)
  const double tau = a.alpha * (double)(*a.smax) / a.block_iter;
  if (threadIdx.x < C) {  // f_j in place of lam_j
    const double s = sqrt(lam[threadIdx.x]);
    lam[threadIdx.x] = (s > 0.0) ? fmax(s - tau, 0.0) / s : 0.0;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < C * C; e += blockDim.x) {
    const int r = e / C, cidx = e % C;
    double2 acc = make_double2(0.0, 0.0);
    for (int j = 0; j < C; j++) {
      const double f = lam[j];
      const double2 t = zmul(V[r * CL_LD + j], zconj(V[cidx * CL_LD + j]));
      acc.x += f * t.x;
      acc.y += f * t.y;
    }
    Mx[r * CL_LD + cidx] = acc;
  }
  __syncthreads();
  // A' = A M, scatter back (src/clear.cpp:780-800): warp per row, lane = coil
  for (int r = warp; r < R; r += nwarp) {
    const int64_t o = row(r);
    const float2 x = lane < C ? (SA ? As[r * C + lane] : a.X[o + lane]) : make_float2(0.f, 0.f);
    double2 acc = make_double2(0.0, 0.0);
    for (int j = 0; j < C; j++) {
      const float xr = __shfl_sync(0xffffffffu, x.x, j), xi = __shfl_sync(0xffffffffu, x.y, j);
      if (lane < C) {
        const double2 m = Mx[j * CL_LD + lane];
        acc.x += (double)xr * m.x - (double)xi * m.y;
        acc.y += (double)xr * m.y + (double)xi * m.x;
      }
    }
    if (lane < C) a.X[o + lane] = make_float2((float)acc.x, (float)acc.y);
  }
}

size_t coil_llr_smem(int T, int C, const int bs[3], bool sa) {
  return sizeof(double2) * 3 * CL_LD * CL_LD + sizeof(double) * (CL_LD + 256) +
         (sa ? sizeof(float2) * (size_t)T * bs[0] * bs[1] * bs[2] * C : 0);
}

constexpr size_t CL_SMEM_MAX = 200 * 1024;

mrg_status coil_llr_launch(CoilLlrArgs &a, int T, int C, const int N[3], const int bs[3], cudaStream_t st) {
  if (C < 1 || C > CL_MAXC) {
    set_error("coil low-rank blocks support 1.." + std::to_string(CL_MAXC) + " coils");
    return MRG_ERR_UNSUPPORTED;
  }
  a.T = T;
  a.C = C;
  a.nvox = (int64_t)N[0] * N[1] * N[2];
  int64_t nblocks = 1;
  for (int d = 0; d < 3; d++) {
    a.N[d] = N[d];
    a.bs[d] = std::min(bs[d], N[d]);  // src/clear.cpp:109-112
    a.nb[d] = N[d] / a.bs[d];
    nblocks *= a.nb[d];
  }
  if (nblocks > INT32_MAX) {
    set_error("too many coil low-rank blocks for one launch");
    return MRG_ERR_UNSUPPORTED;
  }
  static DeviceOnce once;
  MRG_TRY(device_once(once, []() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_llr_coil<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CL_SMEM_MAX));
    MRG_CUDA(cudaFuncSetAttribute(k_llr_coil<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CL_SMEM_MAX));
    return MRG_OK;
  }));
  const bool sa = coil_llr_smem(T, C, a.bs, true) <= CL_SMEM_MAX;
  const size_t smem = coil_llr_smem(T, C, a.bs, sa);
  if (sa)
    k_llr_coil<true><<<(unsigned)nblocks, 256, smem, st>>>(a);
  else
    k_llr_coil<false><<<(unsigned)nblocks, 256, smem, st>>>(a);
  MRG_LAUNCHED();
  return MRG_OK;
}

// sum |R|^2 and sum P conj(R) (src/ArrayTemplates.cpp:462-480) in FP64: per-CTA partials
__global__ void k_clear_dots(const float2 *__restrict__ R, const float2 *__restrict__ P, int64_t n, double *part) {
  __shared__ double s[3][256];
  double rr = 0.0, pr_re = 0.0, pr_im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 r = R[i], p = P[i];
    rr += (double)r.x * r.x + (double)r.y * r.y;
    pr_re += (double)p.x * r.x + (double)p.y * r.y;  // p conj(r)
    pr_im += (double)p.y * r.x - (double)p.x * r.y;
  }
  s[0][threadIdx.x] = rr;
  s[1][threadIdx.x] = pr_re;
  s[2][threadIdx.x] = pr_im;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; k++) s[k][threadIdx.x] += s[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; k++) part[3 * blockIdx.x + k] = s[k][0];
}

// acc (3 doubles) += partials; run as one CTA after each frame's dots
__global__ void k_clear_accum(const double *__restrict__ part, int nblk, double *acc) {
  __shared__ double s[3][256];
  double v[3] = {0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblk; b += blockDim.x)
    for (int k = 0; k < 3; k++) v[k] += part[3 * b + k];
  for (int k = 0; k < 3; k++) s[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; k++) s[k][threadIdx.x] += s[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; k++) acc[k] += s[k][0];
}

// X -= (R^H R / sum P conj R) R  (src/recon_lib.cpp:1111-1147), complex scale in float
__global__ void k_clear_step(float2 *X, const float2 *__restrict__ R, int64_t n, const double *acc) {
  const double rr = acc[0], pre = acc[1], pim = acc[2];
  const double den = pre * pre + pim * pim;
  const double sre = den > 0.0 ? rr * pre / den : 0.0, sim = den > 0.0 ? -rr * pim / den : 0.0;
  const float2 sc = make_float2((float)sre, (float)sim);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 r = R[i];
    const float2 d = make_float2(r.x * sc.x - r.y * sc.y, r.x * sc.y + r.y * sc.x);  // RR *= scale
    X[i] = make_float2(X[i].x - d.x, X[i].y - d.y);
  }
}

}  // namespace

mrg_status clear_dots(const float2 *R, const float2 *P, int64_t n, double *part, int nblk, double *acc,
                      cudaStream_t st) {
  k_clear_dots<<<nblk, 256, 0, st>>>(R, P, n, part);
  MRG_LAUNCHED();
  k_clear_accum<<<1, 256, 0, st>>>(part, nblk, acc);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status clear_step(float2 *X, const float2 *R, int64_t n, const double *acc, cudaStream_t st) {
  k_clear_step<<<grid_blocks(n, 256), 256, 0, st>>>(X, R, n, acc);
  MRG_LAUNCHED();
  return MRG_OK;
}

int64_t coil_llr_blocks(const int N[3], const int bs[3]) {
  int64_t nb = 1;
  for (int d = 0; d < 3; d++) nb *= N[d] / std::min(bs[d], N[d]);
  return nb;
}

mrg_status coil_llr_update(const float2 *X, int T, int C, const int N[3], const int bs[3], float amp, float t2,
                           int iter, double *sig, double *work, float *smax, cudaStream_t st) {
  CoilLlrArgs a;
  memset(&a, 0, sizeof(a));
  a.X = const_cast<float2 *>(X);
  a.mode = 0;
  a.sig = sig;
  MRG_TRY(coil_llr_launch(a, T, C, N, bs, st));
  return llr_median(sig, (int)coil_llr_blocks(N, bs), work, amp, t2, iter, smax, st);
}

mrg_status coil_llr_thresh(float2 *X, int T, int C, const int N[3], const int bs[3], float alpha, int block_iter,
                           const int *shifts, const float *smax, cudaStream_t st) {
  if (alpha == 0.0f) return MRG_OK;  // src/clear.cpp:593-595
  CoilLlrArgs a;
  memset(&a, 0, sizeof(a));
  a.X = X;
  a.mode = 1;
  a.smax = smax;
  a.alpha = (double)alpha;
  a.block_iter = block_iter;
  for (int it = 0; it < block_iter; it++) {
    a.shift = shifts + 3 * it;
    MRG_TRY(coil_llr_launch(a, T, C, N, bs, st));
  }
  return MRG_OK;
}

mrg_status coil_combine(const float2 *X, int T, int C, const int N[3], const int bs[3], float2 *out,
                        cudaStream_t st) {
  CoilLlrArgs a;
  memset(&a, 0, sizeof(a));
  a.X = const_cast<float2 *>(X);
  a.out = out;
  a.mode = 2;
  return coil_llr_launch(a, T, C, N, bs, st);
}

}  // namespace mrg
