// ESPIRiT coil maps: SPIRIT::generateEigenCoils (src/spirit.cpp:137-179) with
// calibrate_ellipsoid (:181-400), prep (:402-439), getcoils (:441-525) and phase_correct
// (:527-550), from per-coil images stored [voxel][coil] (coil innermost).
//
//  1. Only the calibration cube of k-space is used, so the centred inverse FFT of each
//     coil image (ifft, src/ArrayTemplates.cpp:35-88) is evaluated for those outputs
//     alone, as three separable direct DFTs (k_axis_dft): the fftshift sign
//     2((i+j+k)%2)-1 applied before and after the transform is, per axis,
//     (-1)^x (-1)^n, folded into the tables.
//  2. The calibration matrix A (ACS points x kernel points x coils, the reference's
//     row and column order) is gathered, and its SVD is taken by one-sided Jacobi on the
//     columns of A or of A^H, whichever has fewer: per round, one CTA per column pair of
//     a round-robin tournament (every pair once per sweep), sums in double, rotations
//     in float, until no pair is off by more than JAC_TOL (columns far below s0, in the
//     null space of A, are measured against a floor: float cannot orthogonalise them).  The right singular vectors
//     with s >= s0 sqrt(svd_thresh) form the kernels.
//  3. The kernels placed at the centre of each axis and inverse-FFT'd with the chop
//     signs are, per axis, H(x, j) = m(x) m(N/2 + j) e^{2 pi i (N/2 + j) x / N} / sqrt(N),
//     m(i) = 2(i%2)-1, so for each voxel A_x(c, v) = sum_j Hx Hy Hz k(j, c, v) is
//     contracted separably (z for the slice, then y per row, then x per voxel), and
//     M_x = A_x A_x^H is accumulated per voxel.  svd_econ(..., "left")'s U(:, 0) is the
//     dominant eigenvector of M_x: ten squarings of M_x / trace (ratio^1024 of the
//     eigenvalues), a column, then power steps with M_x.  The map is conj(u) times
//     e^{-i arg conj(u_0)} / |u|, which is phase_correct; it does not depend on the phase
//     the eigen-solver returns.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "mrg_internal.h"

namespace mrg {

namespace {

constexpr float JAC_TOL = 4e-6f;  // |a^H b| / (|a| |b|) below which a column pair counts as orthogonal
constexpr int JAC_MAX_SWEEPS = 40;
constexpr double JAC_FLOOR = 1e-6;  // relative to s0^2: columns below 1e-3 s0 count at that norm
constexpr int ESP_XB = 8;  // voxels per CTA in the Gram kernel
constexpr int ESP_VB = 8;  // kernel vectors staged per step

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulcf(float2 a, float2 b) {  // a * conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// out[o][u][i] = scale * sum_l in[o][l][i] tab[l][u]
__global__ void k_axis_dft(const float2 *__restrict__ in, float2 *__restrict__ out, const float2 *__restrict__ tab,
                           int64_t O, int L, int W, int64_t I, float scale) {
  const int64_t n = O * W * I;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % I, t = e / I;
    const int u = (int)(t % W);
    const int64_t o = t / W;
    const float2 *src = in + o * L * I + i;
    float ax = 0.f, ay = 0.f;
    for (int l = 0; l < L; l++) {
      const float2 x = src[(int64_t)l * I], w = tab[(int64_t)l * W + u];
      ax += x.x * w.x - x.y * w.y;
      ay += x.x * w.y + x.y * w.x;
    }
    out[e] = make_float2(ax * scale, ay * scale);
  }
}

// Calibration matrix from the k-space cube Kc[w][v][u][c] (sides 2 cr + 1):
// A(r, c * nk + o) = Kc at rows[r] + kpts[o].  trans = 0: B = A column-major (m x n);
// trans = 1: B = A^H column-major (n x m), i.e. column r = conj(row r of A).
__global__ void k_calib(const float2 *__restrict__ Kc, const int3 *__restrict__ rows, const int3 *__restrict__ kpts,
                        int m, int nk, int C, int3 cr, int trans, float2 *__restrict__ B, float2 *__restrict__ A0) {
  const int n = nk * C;
  const int64_t tot = (int64_t)m * n;
  const int wx = 2 * cr.x + 1, wy = 2 * cr.y + 1;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % m), col = (int)(e / m);
    const int c = col / nk, o = col - c * nk;
    const int3 a = rows[r], k = kpts[o];
    const int u = a.x + k.x + cr.x, v = a.y + k.y + cr.y, w = a.z + k.z + cr.z;
    const float2 val = Kc[(((int64_t)w * wy + v) * wx + u) * C + c];
    if (trans)
      B[(int64_t)r * n + col] = make_float2(val.x, -val.y);
    else
      B[(int64_t)col * m + r] = val;
    if (A0) A0[(int64_t)col * m + r] = val;
  }
}

// One round of the round-robin tournament over k (even) columns of length L: position 0
// stays, positions 1..k-1 rotate by `round`; CTA p pairs positions p and k-1-p.
// A pair counts as off (and is rotated) when |a^H b| >= JAC_TOL sqrt(max(|a|^2, fl) max(|b|^2, fl)),
// fl a floor far below the kept singular values: columns in the numerical null space of A
// cannot be made orthogonal to each other in float, and they are never kept.
__global__ void __launch_bounds__(256) k_jacobi_round(float2 *B, int L, int k, int round, double fl,
                                                      unsigned *maxoff) {
  const int p = blockIdx.x;
  auto col = [&](int pos) { return pos == 0 ? 0 : 1 + (pos - 1 + round) % (k - 1); };
  const int a = col(p), b = col(k - 1 - p);
  float2 *x = B + (int64_t)a * L, *y = B + (int64_t)b * L;
  float sa = 0.f, sb = 0.f, gr = 0.f, gi = 0.f;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const float2 u = x[i], v = y[i];
    sa += u.x * u.x + u.y * u.y;
    sb += v.x * v.x + v.y * v.y;
    gr += u.x * v.x + u.y * v.y;  // conj(u) v
    gi += u.x * v.y - u.y * v.x;
  }
  double d[4] = {sa, sb, gr, gi};
  __shared__ double red[4][8];
  __shared__ float rot[4];  // cs, sn, ph.x, ph.y (cs < 0: skip)
#pragma unroll
  for (int q = 0; q < 4; q++)
    for (int o = 16; o > 0; o >>= 1) d[q] += __shfl_xor_sync(0xffffffffu, d[q], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 4; q++) red[q][wid] = d[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double al = 0, be = 0, re = 0, im = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) al += red[0][w], be += red[1][w], re += red[2][w], im += red[3][w];
    const double ag = sqrt(re * re + im * im);
    rot[0] = -1.f;
    if (al > 0 && be > 0 && ag > 0) {
      const float rel = (float)(ag / sqrt(fmax(al, fl) * fmax(be, fl)));
      atomicMax(maxoff, __float_as_uint(rel));
      if (rel >= JAC_TOL) {
        const double zeta = (be - al) / (2 * ag);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1 + zeta * zeta));
        const double cs = 1 / sqrt(1 + t * t);
        rot[0] = (float)cs;
        rot[1] = (float)(cs * t);
        rot[2] = (float)(re / ag);
        rot[3] = (float)(im / ag);
      }
    }
  }
  __syncthreads();
  const float cs = rot[0];
  if (cs < 0.f) return;
  const float sn = rot[1];
  const float2 ph = make_float2(rot[2], rot[3]);
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const float2 u = x[i], v = cmulcf(y[i], ph);  // y conj(ph)
    x[i] = make_float2(cs * u.x - sn * v.x, cs * u.y - sn * v.y);
    y[i] = cmulf(make_float2(sn * u.x + cs * v.x, sn * u.y + cs * v.y), ph);
  }
}

__global__ void k_colnorm(const float2 *__restrict__ B, int L, int k, double *out) {
  const int j = blockIdx.x;
  if (j >= k) return;
  double s = 0;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const float2 u = B[(int64_t)j * L + i];
    s += (double)u.x * u.x + (double)u.y * u.y;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    out[j] = sqrt(t);
  }
}

// Kernel tensor Vk[v][c][box] (box = jx + bx (jy + by jz), zero outside the kernel
// ellipsoid) from the v-th kept right singular vector of A:
//   trans: column ord[v] of B (= A^H W) is V sigma;  else V = A0^H (column ord[v] of B) / sigma^2.
__global__ void k_kernels(const float2 *__restrict__ B, const float2 *__restrict__ A0, const int *__restrict__ ord,
                          const double *__restrict__ sig, const int *__restrict__ boxidx, int m, int n, int nk, int C,
                          int nV, int nb, int trans, float2 *__restrict__ Vk) {
  const int64_t tot = (int64_t)nV * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int col = (int)(e % n), v = (int)(e / n);
    const int j = ord[v];
    const double s = sig[j];
    double re = 0, im = 0;
    if (trans) {
      const float2 u = B[(int64_t)j * n + col];
      re = u.x / s;
      im = u.y / s;
    } else {
      const float2 *a = A0 + (int64_t)col * m, *bc = B + (int64_t)j * m;
      for (int r = 0; r < m; r++) {  // conj(a) b
        re += (double)a[r].x * bc[r].x + (double)a[r].y * bc[r].y;
        im += (double)a[r].x * bc[r].y - (double)a[r].y * bc[r].x;
      }
      re /= s * s;
      im /= s * s;
    }
    const int c = col / nk, o = col - c * nk;
    Vk[((int64_t)v * C + c) * nb + boxidx[o]] = make_float2((float)re, (float)im);
  }
}

// Kz[v][c][jy][jx] = sum_jz Hz(z, jz) Vk[v][c][jz][jy][jx]
__global__ void k_esp_z(const float2 *__restrict__ Vk, const float2 *__restrict__ Hz, int z, int bx, int by, int bz,
                        int64_t nvc, float2 *__restrict__ Kz) {
  const int pl = bx * by;
  const int64_t tot = nvc * pl;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t vc = e / pl;
    const int q = (int)(e - vc * pl);
    float2 acc = make_float2(0.f, 0.f);
    for (int jz = 0; jz < bz; jz++) {
      const float2 h = Hz[(int64_t)z * bz + jz], kv = Vk[(vc * bz + jz) * pl + q];
      acc.x += h.x * kv.x - h.y * kv.y;
      acc.y += h.x * kv.y + h.y * kv.x;
    }
    Kz[e] = acc;
  }
}

// Kzy[y][v][c][jx] = sum_jy Hy(y, jy) Kz[v][c][jy][jx]
__global__ void k_esp_y(const float2 *__restrict__ Kz, const float2 *__restrict__ Hy, int Ny, int bx, int by,
                        int64_t nvc, float2 *__restrict__ Kzy) {
  const int64_t per = nvc * bx, tot = per * Ny;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(e / per);
    const int64_t r = e - (int64_t)y * per;
    const int64_t vc = r / bx;
    const int jx = (int)(r - vc * bx);
    float2 acc = make_float2(0.f, 0.f);
    for (int jy = 0; jy < by; jy++) {
      const float2 h = Hy[(int64_t)y * by + jy], kv = Kz[(vc * by + jy) * bx + jx];
      acc.x += h.x * kv.x - h.y * kv.y;
      acc.y += h.x * kv.y + h.y * kv.x;
    }
    Kzy[e] = acc;
  }
}

// M_x[c][c'] = sum_v A_x(c, v) conj(A_x(c', v)), A_x(c, v) = sum_jx Hx(x, jx) Kzy[y][v][c][jx],
// for ESP_XB voxels of row y per CTA; entries e = thread + 256 k of the CTA's XB C^2.
__global__ void __launch_bounds__(256) k_esp_gram(const float2 *__restrict__ Kzy, const float2 *__restrict__ Hx, int Nx,
                                                  int nV, int C, int bx, float2 *__restrict__ Mb) {
  __shared__ float2 sK[ESP_VB * 32 * 16];
  __shared__ float2 sA[ESP_XB][ESP_VB][32];
  const int y = blockIdx.y, x0 = blockIdx.x * ESP_XB;
  const int CC = C * C, nent = ESP_XB * CC;
  constexpr int MAXE = ESP_XB * 32 * 32 / 256;
  float2 acc[MAXE];
#pragma unroll
  for (int q = 0; q < MAXE; q++) acc[q] = make_float2(0.f, 0.f);
  const float2 *ky = Kzy + (int64_t)y * nV * C * bx;
  for (int v0 = 0; v0 < nV; v0 += ESP_VB) {
    const int vb = min(ESP_VB, nV - v0);
    __syncthreads();
    for (int e = threadIdx.x; e < vb * C * bx; e += blockDim.x) sK[e] = ky[(int64_t)v0 * C * bx + e];
    __syncthreads();
    for (int e = threadIdx.x; e < ESP_XB * ESP_VB * C; e += blockDim.x) {
      const int c = e % C, t = e / C, vv = t % ESP_VB, xi = t / ESP_VB;
      float2 a = make_float2(0.f, 0.f);
      const int x = x0 + xi;
      if (vv < vb && x < Nx)
        for (int jx = 0; jx < bx; jx++) {
          const float2 h = Hx[(int64_t)x * bx + jx], kv = sK[(vv * C + c) * bx + jx];
          a.x += h.x * kv.x - h.y * kv.y;
          a.y += h.x * kv.y + h.y * kv.x;
        }
      sA[xi][vv][c] = a;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < MAXE; q++) {
      const int e = threadIdx.x + 256 * q;
      if (e < nent) {
        const int xi = e / CC, r = e - xi * CC, c = r / C, c2 = r - c * C;
        float2 s = acc[q];
        for (int vv = 0; vv < vb; vv++) {
          const float2 a = sA[xi][vv][c], b = sA[xi][vv][c2];
          s.x += a.x * b.x + a.y * b.y;
          s.y += a.y * b.x - a.x * b.y;
        }
        acc[q] = s;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < MAXE; q++) {
    const int e = threadIdx.x + 256 * q;
    if (e < nent) {
      const int xi = e / CC, x = x0 + xi;
      if (x < Nx) Mb[((int64_t)y * Nx + x) * CC + (e - xi * CC)] = acc[q];
    }
  }
}

// Dominant eigenvector of each voxel's M (one warp per voxel, lane = row), then the map
// conj(u) e^{-i arg conj(u_0)} / |u| into maps[voxel][c] of slice z.
constexpr int EIG_WARPS = 2;  // 2 x 16.9 KB of shared memory per CTA

__global__ void __launch_bounds__(32 * EIG_WARPS) k_esp_eig(const float2 *__restrict__ Mb, int64_t nvox_slice, int C,
                                                           int64_t out_off, float2 *__restrict__ maps) {
  __shared__ float2 sM[EIG_WARPS][2][32][33];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t vox = (int64_t)blockIdx.x * EIG_WARPS + w;
  if (vox >= nvox_slice) return;
  float2(*P)[33] = sM[w][0];
  float2(*Q)[33] = sM[w][1];
  const float2 *m = Mb + vox * C * C;
  for (int e = lane; e < C * C; e += 32) P[e / C][e % C] = m[e];
  __syncwarp();
  // normalise by the trace (real, non-negative for a Gram matrix)
  auto trace = [&](float2(*X)[33]) {
    float t = lane < C ? X[lane][lane].x : 0.f;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
  };
  float tr = trace(P);
  const bool zero = !(tr > 0.f);
  if (!zero) {
    const float inv = 1.f / tr;
    if (lane < C)
      for (int j = 0; j < C; j++) P[lane][j] = make_float2(P[lane][j].x * inv, P[lane][j].y * inv);
  }
  __syncwarp();
  // keep M / tr in registers (row `lane`) for the power steps
  float2 row[32];
#pragma unroll
  for (int j = 0; j < 32; j++) row[j] = (lane < C && j < C) ? P[lane][j] : make_float2(0.f, 0.f);
  if (!zero) {
    for (int sq = 0; sq < 10; sq++) {  // P <- P^2 / tr(P^2)
      if (lane < C)
        for (int j = 0; j < C; j++) {
          float2 s = make_float2(0.f, 0.f);
          for (int q = 0; q < C; q++) {
            const float2 a = P[lane][q], b = P[q][j];
            s.x += a.x * b.x - a.y * b.y;
            s.y += a.x * b.y + a.y * b.x;
          }
          Q[lane][j] = s;
        }
      __syncwarp();
      const float t2 = trace(Q);
      const float inv = t2 > 0.f ? 1.f / t2 : 0.f;
      if (lane < C)
        for (int j = 0; j < C; j++) P[lane][j] = make_float2(Q[lane][j].x * inv, Q[lane][j].y * inv);
      __syncwarp();
    }
  }
  // u = the column of P with the largest diagonal entry, then power steps with M
  float d = (lane < C) ? P[lane][lane].x : -1.f;
  int jm = lane;
  for (int o = 16; o > 0; o >>= 1) {
    const float d2 = __shfl_xor_sync(0xffffffffu, d, o);
    const int j2 = __shfl_xor_sync(0xffffffffu, jm, o);
    if (d2 > d || (d2 == d && j2 < jm)) d = d2, jm = j2;
  }
  float2 u = (lane < C) ? (zero ? make_float2(lane == 0 ? 1.f : 0.f, 0.f) : P[lane][jm]) : make_float2(0.f, 0.f);
  for (int it = 0; it < 4 && !zero; it++) {
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 32; q++) {
      const float ux = __shfl_sync(0xffffffffu, u.x, q), uy = __shfl_sync(0xffffffffu, u.y, q);
      s.x += row[q].x * ux - row[q].y * uy;
      s.y += row[q].x * uy + row[q].y * ux;
    }
    float nn = s.x * s.x + s.y * s.y;
    for (int o = 16; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
    if (!(nn > 0.f)) break;
    const float inv = rsqrtf(nn);
    u = make_float2(s.x * inv, s.y * inv);
  }
  // LR(c) = conj(u_c); phase_correct: x polar(1, -arg(LR(0))) / sqrt(sum |LR|^2)
  float mag = u.x * u.x + u.y * u.y;
  for (int o = 16; o > 0; o >>= 1) mag += __shfl_xor_sync(0xffffffffu, mag, o);
  const float u0x = __shfl_sync(0xffffffffu, u.x, 0), u0y = __shfl_sync(0xffffffffu, u.y, 0);
  const float a0 = atan2f(-u0y, u0x);  // arg(conj(u_0))
  float sa, ca;
  sincosf(-a0, &sa, &ca);
  const float inv = mag > 0.f ? 1.f / sqrtf(mag) : 0.f;
  const float2 ci = make_float2(ca * inv, sa * inv);
  if (lane < C) maps[(out_off + vox) * C + lane] = cmulf(make_float2(u.x, -u.y), ci);
}

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 32)); }

}  // namespace

mrg_status espirit_maps(const float2 *img, int C, const int N[3], const EspiritParams &q, float2 *maps, int *nV_out,
                        cudaStream_t st) {
  const int64_t nx = N[0], ny = N[1], nz = N[2], nvox = nx * ny * nz;
  if (C < 1 || C > 32) {
    set_error("ESPIRiT maps support 1..32 coils");
    return MRG_ERR_UNSUPPORTED;
  }
  // init (src/spirit.cpp:36-64)
  float kf[3];
  int kr[3], cr[3];
  for (int d = 0; d < 3; d++) {
    kf[d] = q.kr_f[d];
    kr[d] = (int)std::ceil(kf[d]);
    cr[d] = q.cr[d];
  }
  if (nz == 1) kr[2] = 0, cr[2] = 0;
  int ce[3];
  for (int d = 0; d < 3; d++) {
    ce[d] = cr[d] - kr[d];
    const bool flat = (d == 2 && nz == 1);
    if (kr[d] > 7) {  // the Gram kernel stages 2 kr + 1 <= 16 taps per coil and vector
      set_error("ESPIRiT kernel radius must be at most 7");
      return MRG_ERR_INVALID;
    }
    if (!flat && (kr[d] < 0 || ce[d] < 1 || 2 * cr[d] + 1 > N[d] || N[d] / 2 + cr[d] >= N[d])) {
      set_error("ESPIRiT: calibration radius must exceed the kernel radius and fit the image");
      return MRG_ERR_INVALID;
    }
  }
  // rows (ACS points) and kernel points in the reference's order
  std::vector<int3> rows, kpts;
  auto acs = [&](int ix, int iy, int iz) {
    if (q.square) return true;
    float rad;
    if (ce[2] == 0) rad = (float)(ix * ix) / (ce[0] * ce[0]) + (float)(iy * iy) / (ce[1] * ce[1]);
    else rad = (float)(ix * ix) / (ce[0] * ce[0]) + (float)(iy * iy) / (ce[1] * ce[1]) + (float)(iz * iz) / (ce[2] * ce[2]);
    return !(rad > 1);
  };
  auto kin = [&](int jx, int jy, int jz) {
    if (q.square) return true;
    float krad;
    if (kf[2] == 0) krad = (float)(jx * jx) / (kf[0] * kf[0]) + (float)(jy * jy) / (kf[1] * kf[1]);
    else krad = (float)(jx * jx) / (kf[0] * kf[0]) + (float)(jy * jy) / (kf[1] * kf[1]) + (float)(jz * jz) / (kf[2] * kf[2]);
    return krad <= 1;
  };
  for (int iz = -ce[2]; iz <= ce[2]; iz++)
    for (int iy = -ce[1]; iy <= ce[1]; iy++)
      for (int ix = -ce[0]; ix <= ce[0]; ix++)
        if (acs(ix, iy, iz)) rows.push_back(make_int3(ix, iy, iz));
  const int bx = 2 * kr[0] + 1, by = 2 * kr[1] + 1, bz = 2 * kr[2] + 1, nb = bx * by * bz;
  std::vector<int> boxidx;
  for (int jz = -kr[2]; jz <= kr[2]; jz++)
    for (int jy = -kr[1]; jy <= kr[1]; jy++)
      for (int jx = -kr[0]; jx <= kr[0]; jx++)
        if (kin(jx, jy, jz)) {
          kpts.push_back(make_int3(jx, jy, jz));
          boxidx.push_back((jx + kr[0]) + bx * ((jy + kr[1]) + by * (jz + kr[2])));
        }
  const int m = (int)rows.size(), nk = (int)kpts.size(), n = nk * C;
  if (m < 1 || nk < 1) {
    set_error("ESPIRiT: empty calibration region or kernel");
    return MRG_ERR_INVALID;
  }
  const bool trans = m < n;  // Jacobi on the columns of A^H when A has more columns than rows
  const int kc = trans ? m : n, L = trans ? n : m, keven = kc + (kc & 1);
  const int W[3] = {2 * cr[0] + 1, 2 * cr[1] + 1, 2 * cr[2] + 1};
  // per-axis tables (double on the host): DFT to the calibration cube and H for the maps
  std::vector<float2> tab[3], H[3];
  for (int d = 0; d < 3; d++) {
    const int NN = N[d];
    tab[d].resize((size_t)NN * W[d]);
    for (int x = 0; x < NN; x++)
      for (int u = 0; u < W[d]; u++) {
        const int64_t nn = NN / 2 - cr[d] + u;
        const double a = 2.0 * M_PI * (double)((nn * x) % NN) / (double)NN;
        const double sg = ((x + nn) % 2) ? -1.0 : 1.0;
        tab[d][(size_t)x * W[d] + u] = make_float2((float)(sg * std::cos(a)), (float)(sg * std::sin(a)));
      }
    const int bd = 2 * kr[d] + 1;
    H[d].resize((size_t)NN * bd);
    const double sc = (double)(float)(1. / std::sqrt((float)NN));
    for (int x = 0; x < NN; x++)
      for (int j = 0; j < bd; j++) {
        const int64_t nn = NN / 2 + (j - kr[d]);
        const double a = 2.0 * M_PI * (double)((nn * x) % NN) / (double)NN;
        const double sg = ((x + nn) % 2) ? -1.0 : 1.0;  // m(x) m(nn)
        H[d][(size_t)x * bd + j] = make_float2((float)(sg * sc * std::cos(a)), (float)(sg * sc * std::sin(a)));
      }
  }
  struct Bufs {
    std::vector<void *> p;
    void *get(size_t bytes, mrg_status &s) {
      void *x = nullptr;
      if (s == MRG_OK && cudaMalloc(&x, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        set_error("ESPIRiT: out of device memory");
        s = MRG_ERR_NOMEM;
        return nullptr;
      }
      p.push_back(x);
      return x;
    }
    ~Bufs() {
      for (void *x : p) cudaFree(x);
    }
  } b;
  mrg_status s = MRG_OK;
  float2 *dtab[3], *dH[3];
  for (int d = 0; d < 3; d++) {
    dtab[d] = (float2 *)b.get(sizeof(float2) * tab[d].size(), s);
    dH[d] = (float2 *)b.get(sizeof(float2) * H[d].size(), s);
  }
  float2 *T1 = (float2 *)b.get(sizeof(float2) * (size_t)nz * ny * W[0] * C, s);
  float2 *T2 = (float2 *)b.get(sizeof(float2) * (size_t)nz * W[1] * W[0] * C, s);
  float2 *Kc = (float2 *)b.get(sizeof(float2) * (size_t)W[2] * W[1] * W[0] * C, s);
  int3 *drows = (int3 *)b.get(sizeof(int3) * rows.size(), s);
  int3 *dkp = (int3 *)b.get(sizeof(int3) * kpts.size(), s);
  int *dbox = (int *)b.get(sizeof(int) * boxidx.size(), s);
  float2 *B = (float2 *)b.get(sizeof(float2) * (size_t)L * keven, s);
  float2 *A0 = trans ? nullptr : (float2 *)b.get(sizeof(float2) * (size_t)m * n, s);
  double *sig = (double *)b.get(sizeof(double) * keven, s);
  unsigned *dmax = (unsigned *)b.get(sizeof(unsigned), s);
  MRG_TRY(s);
  for (int d = 0; d < 3; d++) {
    MRG_CUDA(cudaMemcpyAsync(dtab[d], tab[d].data(), sizeof(float2) * tab[d].size(), cudaMemcpyHostToDevice, st));
    MRG_CUDA(cudaMemcpyAsync(dH[d], H[d].data(), sizeof(float2) * H[d].size(), cudaMemcpyHostToDevice, st));
  }
  MRG_CUDA(cudaMemcpyAsync(drows, rows.data(), sizeof(int3) * rows.size(), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaMemcpyAsync(dkp, kpts.data(), sizeof(int3) * kpts.size(), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaMemcpyAsync(dbox, boxidx.data(), sizeof(int) * boxidx.size(), cudaMemcpyHostToDevice, st));
  // 1. calibration cube of the centred inverse FFT (x, then y, then z; one float scale)
  const float scale = (float)(1.0 / std::sqrt((float)nz * (float)ny * (float)nx));
  int64_t ne = nz * ny * W[0] * C;
  k_axis_dft<<<grid_for(ne), 256, 0, st>>>(img, T1, dtab[0], nz * ny, (int)nx, W[0], C, 1.0f);
  MRG_LAUNCHED();
  ne = nz * W[1] * W[0] * C;
  k_axis_dft<<<grid_for(ne), 256, 0, st>>>(T1, T2, dtab[1], nz, (int)ny, W[1], (int64_t)W[0] * C, 1.0f);
  MRG_LAUNCHED();
  ne = (int64_t)W[2] * W[1] * W[0] * C;
  k_axis_dft<<<grid_for(ne), 256, 0, st>>>(T2, Kc, dtab[2], 1, (int)nz, W[2], (int64_t)W[1] * W[0] * C, scale);
  MRG_LAUNCHED();
  // 2. calibration matrix and its SVD
  MRG_CUDA(cudaMemsetAsync(B, 0, sizeof(float2) * (size_t)L * keven, st));
  const int3 cr3 = make_int3(cr[0], cr[1], cr[2]);
  k_calib<<<grid_for((int64_t)m * n), 256, 0, st>>>(Kc, drows, dkp, m, nk, C, cr3, trans ? 1 : 0, B, A0);
  MRG_LAUNCHED();
  int sweeps = 0;
  if (keven >= 2) {
    // floor of the pair test: JAC_FLOOR x the largest column norm^2 (<= s0^2)
    k_colnorm<<<keven, 256, 0, st>>>(B, L, keven, sig);
    MRG_LAUNCHED();
    std::vector<double> h0(keven);
    MRG_CUDA(cudaMemcpyAsync(h0.data(), sig, sizeof(double) * keven, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
    const double cmax = *std::max_element(h0.begin(), h0.end());
    const double fl = JAC_FLOOR * cmax * cmax;
    for (; sweeps < JAC_MAX_SWEEPS; sweeps++) {
      MRG_CUDA(cudaMemsetAsync(dmax, 0, sizeof(unsigned), st));
      for (int r = 0; r < keven - 1; r++) {
        k_jacobi_round<<<keven / 2, 256, 0, st>>>(B, L, keven, r, fl, dmax);
        MRG_LAUNCHED();
      }
      unsigned hm = 0;
      MRG_CUDA(cudaMemcpyAsync(&hm, dmax, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
      MRG_CUDA(cudaStreamSynchronize(st));
      float off;
      memcpy(&off, &hm, sizeof(float));
      if (off < JAC_TOL) break;
    }
  }
  k_colnorm<<<keven, 256, 0, st>>>(B, L, keven, sig);
  MRG_LAUNCHED();
  std::vector<double> hs(keven);
  MRG_CUDA(cudaMemcpyAsync(hs.data(), sig, sizeof(double) * keven, cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  std::vector<int> ord(keven);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return hs[a] > hs[c]; });
  // nV: s >= s(0) sqrt(svd_thresh) among the min(m, n) singular values (src/spirit.cpp:339-347)
  const float thresh = (float)(hs[ord[0]] * std::sqrt(q.svd_thresh));
  int nV = 0;
  for (int j = 0; j < std::min(m, n); j++)
    if (hs[ord[j]] >= thresh && hs[ord[j]] > 0) nV++;
  if (nV_out) *nV_out = nV;
  if (q.sv_out)
    for (int j = 0; j < std::min(std::min(m, n), q.sv_cap); j++) q.sv_out[j] = hs[ord[j]];
  if (nV == 0) {
    set_error("ESPIRiT: calibration data are all zero");
    return MRG_ERR_INVALID;
  }
  int *dord = (int *)b.get(sizeof(int) * nV, s);
  float2 *Vk = (float2 *)b.get(sizeof(float2) * (size_t)nV * C * nb, s);
  const int64_t nvc = (int64_t)nV * C;
  float2 *Kz = (float2 *)b.get(sizeof(float2) * (size_t)nvc * bx * by, s);
  float2 *Kzy = (float2 *)b.get(sizeof(float2) * (size_t)ny * nvc * bx, s);
  float2 *Mb = (float2 *)b.get(sizeof(float2) * (size_t)nx * ny * C * C, s);
  MRG_TRY(s);
  MRG_CUDA(cudaMemcpyAsync(dord, ord.data(), sizeof(int) * nV, cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaMemsetAsync(Vk, 0, sizeof(float2) * (size_t)nV * C * nb, st));
  k_kernels<<<grid_for((int64_t)nV * n), 256, 0, st>>>(B, A0, dord, sig, dbox, m, n, nk, C, nV, nb, trans ? 1 : 0, Vk);
  MRG_LAUNCHED();
  // 3. per slice: kernels to image space, M_x per voxel, dominant eigenvector, phase
  const dim3 gg((unsigned)((nx + ESP_XB - 1) / ESP_XB), (unsigned)ny);
  for (int64_t z = 0; z < nz; z++) {
    k_esp_z<<<grid_for(nvc * bx * by), 256, 0, st>>>(Vk, dH[2], (int)z, bx, by, bz, nvc, Kz);
    MRG_LAUNCHED();
    k_esp_y<<<grid_for(ny * nvc * bx), 256, 0, st>>>(Kz, dH[1], (int)ny, bx, by, nvc, Kzy);
    MRG_LAUNCHED();
    k_esp_gram<<<gg, 256, 0, st>>>(Kzy, dH[0], (int)nx, nV, C, bx, Mb);
    MRG_LAUNCHED();
    k_esp_eig<<<(unsigned)((nx * ny + EIG_WARPS - 1) / EIG_WARPS), 32 * EIG_WARPS, 0, st>>>(Mb, nx * ny, C,
                                                                                       z * nx * ny, maps);
    MRG_LAUNCHED();
  }
  MRG_CUDA(cudaStreamSynchronize(st));
  (void)nvox;
  (void)sweeps;
  return MRG_OK;
}

}  // namespace mrg
