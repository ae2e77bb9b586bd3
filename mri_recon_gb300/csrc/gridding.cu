// Kaiser-Bessel gridding (E^H front end) and ungridding (E back end).
//
// Arithmetic follows gridFFT::chop_grid_forward / chop_grid_backward
// (src/gridFFT.cpp:1009-1322): grid position dk = k*grid + S/2 in float, taps
// ceil(dk - dwin) .. floor(dk + dwin) clipped to [0, S-1] (no wrap), tap weight
// = LUT(|600*(dk - l)|) linearly interpolated, times the chop sign
// (2*(l%2) - 1) per axis; E^H scatters data*kw*exp(-|k|^2/(2 k_rad^2)).
//
// GB300 layout: all coils of a sample are adjacent ([sample][coil] for k-space,
// [z][y][x][coil] for the grid), so one weight computation serves every coil
// and a group of G lanes (lane = coil) moves C contiguous complex values per tap.
//
// Samples are sorted by the grid tile (B^3 points) that holds their centre.
// Ungridding walks samples in that order (tile-local gathers hit L1/L2).
// Gridding is owner-computes: each tile is produced by the work items that own
// it, from the list of every sample whose kernel support touches the tile, so
// the accumulation runs in shared memory with shared atomics and the tile is
// written to HBM once with plain stores; only tiles whose pair list is split
// across several items (the dense k-space centre) use global atomics.
#include <algorithm>

#include "mrg_internal.h"

namespace mrg {

__device__ __forceinline__ float tap_w(const float *__restrict__ lut, float gmod, float dk, int l) {
  const float del = fabsf(__fmul_rn(gmod, __fsub_rn(dk, (float)l)));
  const int i0 = (int)del;
  const float f = __fsub_rn(del, (float)i0);
  const float w = __ldg(lut + i0) * (1.0f - f) + __ldg(lut + i0 + 1) * f;
  return (l & 1) ? w : -w;
}

__device__ __forceinline__ void tap_range(const GridConst &g, int d, float dk, int &s, int &e) {
  s = max((int)ceilf(__fsub_rn(dk, g.dwin[d])), 0);
  e = min((int)floorf(__fadd_rn(dk, g.dwin[d])), g.S[d] - 1);
}

// ---------------------------------------------------------------------------
// trajectory setup
// ---------------------------------------------------------------------------
__global__ void k_traj_prep(GridConst g, const float *__restrict__ kx, const float *__restrict__ ky,
                            const float *__restrict__ kz, const float *__restrict__ kw, int64_t M, float4 *pos,
                            float *tap, int *key, int *cnt, int ntiles) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const float k[3] = {kx[i], ky[i], kz[i]};
    const float w = kw[i];
    bool ok = (w != 0.0f);
    float dk[3];
    int cell[3];
    for (int d = 0; d < 3; d++) {
      dk[d] = __fadd_rn(__fmul_rn(k[d], g.grid[d]), g.cen[d]);
      int s, e;
      tap_range(g, d, dk[d], s, e);
      ok = ok && !(s >= g.S[d] || e < 0);
      int c = (int)floorf(dk[d]);
      c = min(max(c, 0), g.S[d] - 1);
      cell[d] = c / g.B;
    }
    // kr = kx*kx + ky*ky + kz*kz accumulated in float, taper in double (src/gridFFT.cpp:1096-1108)
    float kr = 0.0f;
    kr = __fadd_rn(kr, __fmul_rn(k[0], k[0]));
    kr = __fadd_rn(kr, __fmul_rn(k[1], k[1]));
    kr = __fadd_rn(kr, __fmul_rn(k[2], k[2]));
    const float tp = (float)exp(-(double)kr / (2.0 * (double)g.k_rad * (double)g.k_rad));
    const int kk = ok ? (cell[2] * g.nt[1] + cell[1]) * g.nt[0] + cell[0] : ntiles;
    pos[i] = make_float4(dk[0], dk[1], dk[2], w);
    tap[i] = tp;
    key[i] = kk;
    atomicAdd(&cnt[kk], 1);
  }
}

// Exclusive scan of n ints (single CTA of 1024 threads, contiguous chunks).
__global__ void k_scan(const int *__restrict__ in, int *out, int n) {
  __shared__ long long part[1024];
  const int T = blockDim.x, t = threadIdx.x;
  const int per = (n + T - 1) / T;
  const int a = min(n, t * per), b = min(n, a + per);
  long long s = 0;
  for (int k = a; k < b; k++) s += in[k];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    long long run = 0;
    for (int k = 0; k < T; k++) {
      long long v = part[k];
      part[k] = run;
      run += v;
    }
  }
  __syncthreads();
  long long run = part[t];
  for (int k = a; k < b; k++) {
    int v = in[k];
    out[k] = (int)run;
    run += v;
  }
  if (b == n && a < b) out[n] = (int)run;
  if (n == 0 && t == 0) out[0] = 0;
}

__global__ void k_traj_sort(int64_t M, const int *__restrict__ key, const int *__restrict__ off, int *cur,
                            const float4 *__restrict__ pos, const float *__restrict__ tap, float4 *spos, float *stap,
                            int *perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = key[i];
    const int s = off[k] + atomicAdd(&cur[k], 1);
    spos[s] = pos[i];
    stap[s] = tap[i];
    perm[s] = (int)i;
  }
}

template <bool FILL>
__global__ void k_pairs(GridConst g, int nvalid, const float4 *__restrict__ spos, int *pcnt, const int *__restrict__ poff,
                        int *pcur, int *pairs) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nvalid; s += gridDim.x * blockDim.x) {
    const float4 p = spos[s];
    const float dk[3] = {p.x, p.y, p.z};
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      int a, b;
      tap_range(g, d, dk[d], a, b);
      lo[d] = a / g.B;
      hi[d] = b / g.B;
    }
    for (int tz = lo[2]; tz <= hi[2]; tz++)
      for (int ty = lo[1]; ty <= hi[1]; ty++)
        for (int tx = lo[0]; tx <= hi[0]; tx++) {
          const int tile = (tz * g.nt[1] + ty) * g.nt[0] + tx;
          if (FILL) pairs[poff[tile] + atomicAdd(&pcur[tile], 1)] = s;
          else atomicAdd(&pcnt[tile], 1);
        }
  }
}

__global__ void k_item_count(int ntiles, const int *__restrict__ pcnt, int maxp, int *icnt) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
    icnt[t] = max(1, (pcnt[t] + maxp - 1) / maxp);
}

__global__ void k_item_fill(int ntiles, const int *__restrict__ pcnt, const int *__restrict__ poff,
                            const int *__restrict__ icnt, const int *__restrict__ ioff, int maxp, int4 *items,
                            int *split, int *nsplit) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
    const int n = icnt[t];
    for (int k = 0; k < n; k++) {
      const int p0 = poff[t] + k * maxp;
      const int p1 = min(poff[t] + pcnt[t], p0 + maxp);
      items[ioff[t] + k] = make_int4(t, p0, p1, n > 1 ? 1 : 0);
    }
    if (n > 1) split[atomicAdd(nsplit, 1)] = t;
  }
}

static int grid_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 64) b = 152 * 64;
  return (int)b;
}

template <typename T>
static mrg_status dalloc(T **p, int64_t n) {
  *p = nullptr;
  if (n <= 0) n = 1;
  MRG_CUDA(cudaMalloc((void **)p, sizeof(T) * (size_t)n));
  return MRG_OK;
}

void traj_free(FrameTraj &ft) {
  cudaFree(ft.spos);
  cudaFree(ft.stap);
  cudaFree(ft.perm);
  cudaFree(ft.pairs);
  cudaFree(ft.items);
  cudaFree(ft.split_tiles);
  cudaFree(ft.dsorted);
  ft = FrameTraj();
}

mrg_status traj_setup(const GridConst &gc, FrameTraj &ft, const float *kx, const float *ky, const float *kz,
                      const float *kw, int64_t M, int max_pairs, cudaStream_t st) {
  traj_free(ft);
  if (M <= 0 || M >= (int64_t)1 << 31) {
    set_error("trajectory length must be in [1, 2^31)");
    return MRG_ERR_INVALID;
  }
  const int ntiles = gc.nt[0] * gc.nt[1] * gc.nt[2];
  ft.M = M;
  float4 *pos = nullptr;
  float *tap = nullptr;
  int *key = nullptr, *cnt = nullptr, *off = nullptr, *cur = nullptr;
  int *pcnt = nullptr, *poff = nullptr, *pcur = nullptr, *icnt = nullptr, *ioff = nullptr, *nsplit = nullptr;
  mrg_status rs = MRG_OK;
  auto cleanup = [&]() {
    cudaFree(pos); cudaFree(tap); cudaFree(key); cudaFree(cnt); cudaFree(off); cudaFree(cur);
    cudaFree(pcnt); cudaFree(poff); cudaFree(pcur); cudaFree(icnt); cudaFree(ioff); cudaFree(nsplit);
  };
#define SETUP_TRY(x)         \
  do {                       \
    rs = (x);                \
    if (rs != MRG_OK) {      \
      cleanup();             \
      traj_free(ft);         \
      return rs;             \
    }                        \
  } while (0)
  SETUP_TRY(dalloc(&pos, M));
  SETUP_TRY(dalloc(&tap, M));
  SETUP_TRY(dalloc(&key, M));
  SETUP_TRY(dalloc(&cnt, ntiles + 1));
  SETUP_TRY(dalloc(&off, ntiles + 2));
  SETUP_TRY(dalloc(&cur, ntiles + 1));
  SETUP_TRY(dalloc(&ft.spos, M));
  SETUP_TRY(dalloc(&ft.stap, M));
  SETUP_TRY(dalloc(&ft.perm, M));
  SETUP_TRY(launch_zero(cnt, sizeof(int) * (ntiles + 1), st));
  SETUP_TRY(launch_zero(cur, sizeof(int) * (ntiles + 1), st));
  k_traj_prep<<<grid_blocks(M, 256), 256, 0, st>>>(gc, kx, ky, kz, kw, M, pos, tap, key, cnt, ntiles);
  SETUP_TRY(cudaGetLastError() == cudaSuccess ? MRG_OK : MRG_ERR_CUDA);
  count_launch();
  k_scan<<<1, 1024, 0, st>>>(cnt, off, ntiles + 1);
  count_launch();
  k_traj_sort<<<grid_blocks(M, 256), 256, 0, st>>>(M, key, off, cur, pos, tap, ft.spos, ft.stap, ft.perm);
  count_launch();
  int nvalid = 0;
  if (cudaMemcpyAsync(&nvalid, off + ntiles, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    set_error(std::string("trajectory sort failed: ") + cudaGetErrorString(cudaGetLastError()));
    cleanup();
    traj_free(ft);
    return MRG_ERR_CUDA;
  }
  ft.nvalid = nvalid;

  // (sample, tile) pairs
  SETUP_TRY(dalloc(&pcnt, ntiles + 1));
  SETUP_TRY(dalloc(&poff, ntiles + 2));
  SETUP_TRY(dalloc(&pcur, ntiles + 1));
  SETUP_TRY(launch_zero(pcnt, sizeof(int) * (ntiles + 1), st));
  SETUP_TRY(launch_zero(pcur, sizeof(int) * (ntiles + 1), st));
  k_pairs<false><<<grid_blocks(nvalid, 256), 256, 0, st>>>(gc, nvalid, ft.spos, pcnt, nullptr, nullptr, nullptr);
  count_launch();
  k_scan<<<1, 1024, 0, st>>>(pcnt, poff, ntiles);
  count_launch();
  int npairs = 0;
  if (cudaMemcpyAsync(&npairs, poff + ntiles, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    set_error("pair count failed");
    cleanup();
    traj_free(ft);
    return MRG_ERR_CUDA;
  }
  ft.npairs = npairs;
  SETUP_TRY(dalloc(&ft.pairs, npairs));
  k_pairs<true><<<grid_blocks(nvalid, 256), 256, 0, st>>>(gc, nvalid, ft.spos, nullptr, poff, pcur, ft.pairs);
  count_launch();

  // work items: at most max_pairs pairs each; every tile gets >= 1 item
  SETUP_TRY(dalloc(&icnt, ntiles + 1));
  SETUP_TRY(dalloc(&ioff, ntiles + 2));
  SETUP_TRY(dalloc(&nsplit, 1));
  SETUP_TRY(launch_zero(nsplit, sizeof(int), st));
  k_item_count<<<grid_blocks(ntiles, 256), 256, 0, st>>>(ntiles, pcnt, max_pairs, icnt);
  count_launch();
  k_scan<<<1, 1024, 0, st>>>(icnt, ioff, ntiles);
  count_launch();
  int nitems = 0;
  if (cudaMemcpyAsync(&nitems, ioff + ntiles, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    set_error("item count failed");
    cleanup();
    traj_free(ft);
    return MRG_ERR_CUDA;
  }
  ft.nitems = nitems;
  SETUP_TRY(dalloc(&ft.items, nitems));
  SETUP_TRY(dalloc(&ft.split_tiles, ntiles));
  k_item_fill<<<grid_blocks(ntiles, 256), 256, 0, st>>>(ntiles, pcnt, poff, icnt, ioff, max_pairs, ft.items,
                                                        ft.split_tiles, nsplit);
  count_launch();
  int ns = 0;
  if (cudaMemcpyAsync(&ns, nsplit, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    set_error("item fill failed");
    cleanup();
    traj_free(ft);
    return MRG_ERR_CUDA;
  }
  ft.nsplit = ns;
  cleanup();
#undef SETUP_TRY
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// ungridding: y[s][c] = sum_taps w * grid[tap][c]  (- diff[s][c])
// ---------------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(256) k_ungrid(const GridConst g, int nvalid, const float4 *__restrict__ spos,
                                               const float2 *__restrict__ grid, const float2 *__restrict__ diff,
                                               float2 *__restrict__ y) {
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int lane = threadIdx.x % G;
  if (gid >= nvalid) return;
  const float4 p = spos[gid];
  int xs, xe, ys, ye, zs, ze;
  tap_range(g, 0, p.x, xs, xe);
  tap_range(g, 1, p.y, ys, ye);
  tap_range(g, 2, p.z, zs, ze);
  float wx[6];
#pragma unroll
  for (int a = 0; a < 6; a++) wx[a] = (xs + a <= xe) ? tap_w(g.lut[0], g.gmod[0], p.x, xs + a) : 0.0f;
  const int C = g.C;
  const int64_t S0 = g.S[0], S1 = g.S[1];
  for (int cb = 0; cb < C; cb += G) {
    const int c = cb + lane;
    if (c >= C) break;
    float2 acc = make_float2(0.f, 0.f);
    for (int lz = zs; lz <= ze; lz++) {
      const float wz = tap_w(g.lut[2], g.gmod[2], p.z, lz);
      for (int ly = ys; ly <= ye; ly++) {
        const float wzy = wz * tap_w(g.lut[1], g.gmod[1], p.y, ly);
        const float2 *row = grid + (((int64_t)lz * S1 + ly) * S0 + xs) * C + c;
#pragma unroll
        for (int a = 0; a < 6; a++) {
          if (xs + a <= xe) {
            const float w = wzy * wx[a];
            const float2 v = __ldg(row + (int64_t)a * C);
            acc.x += w * v.x;
            acc.y += w * v.y;
          }
        }
      }
    }
    const int64_t o = gid * C + c;
    if (diff) {
      const float2 d = diff[o];
      acc.x -= d.x;
      acc.y -= d.y;
    }
    y[o] = acc;
  }
}

mrg_status launch_ungrid(const GridConst &gc, const FrameTraj &ft, const float2 *grid, const float2 *diff, float2 *y,
                         cudaStream_t st) {
  if (ft.nvalid == 0) return MRG_OK;
  int G = 1;
  while (G < gc.C && G < 32) G *= 2;
  const int64_t threads = (int64_t)ft.nvalid * G;
  const int blocks = (int)((threads + 255) / 256);
  switch (G) {
    case 1: k_ungrid<1><<<blocks, 256, 0, st>>>(gc, ft.nvalid, ft.spos, grid, diff, y); break;
    case 2: k_ungrid<2><<<blocks, 256, 0, st>>>(gc, ft.nvalid, ft.spos, grid, diff, y); break;
    case 4: k_ungrid<4><<<blocks, 256, 0, st>>>(gc, ft.nvalid, ft.spos, grid, diff, y); break;
    case 8: k_ungrid<8><<<blocks, 256, 0, st>>>(gc, ft.nvalid, ft.spos, grid, diff, y); break;
    case 16: k_ungrid<16><<<blocks, 256, 0, st>>>(gc, ft.nvalid, ft.spos, grid, diff, y); break;
    default: k_ungrid<32><<<blocks, 256, 0, st>>>(gc, ft.nvalid, ft.spos, grid, diff, y); break;
  }
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// gridding: owner-computes tiles, shared-memory accumulation
// ---------------------------------------------------------------------------
__global__ void k_zero_tiles(const GridConst g, const int *__restrict__ tiles, int n, float2 *grid) {
  const int B = g.B, C = g.C;
  const int per = B * B * B * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n * per;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int t = tiles[e / per];
    int r = (int)(e % per);
    const int c = r % C;
    r /= C;
    const int px = r % B, py = (r / B) % B, pz = r / (B * B);
    const int tx = t % g.nt[0], ty = (t / g.nt[0]) % g.nt[1], tz = t / (g.nt[0] * g.nt[1]);
    const int64_t gi = ((((int64_t)(tz * B + pz)) * g.S[1] + (ty * B + py)) * g.S[0] + (tx * B + px)) * C + c;
    grid[gi] = make_float2(0.f, 0.f);
  }
}

template <int G>
__global__ void __launch_bounds__(256) k_grid(const GridConst g, const int4 *__restrict__ items,
                                             const int *__restrict__ pairs, const float4 *__restrict__ spos,
                                             const float *__restrict__ stap, const float2 *__restrict__ y,
                                             float2 *__restrict__ grid) {
  extern __shared__ float tile[];  // [B^3][2][G]
  const int B = g.B, B3 = B * B * B;
  const int C = g.C;
  const int4 it = items[blockIdx.x];
  const int cb = blockIdx.y * G;
  for (int e = threadIdx.x; e < B3 * 2 * G; e += blockDim.x) tile[e] = 0.0f;
  const int tx = it.x % g.nt[0], ty = (it.x / g.nt[0]) % g.nt[1], tz = it.x / (g.nt[0] * g.nt[1]);
  const int x0 = tx * B, y0 = ty * B, z0 = tz * B;
  __syncthreads();

  const int lane = threadIdx.x % G;
  const int grp = threadIdx.x / G, ngrp = blockDim.x / G;
  const int c = cb + lane;
  for (int q = it.y + grp; q < it.z; q += ngrp) {
    const int s = pairs[q];
    const float4 p = spos[s];
    int xs, xe, ys, ye, zs, ze;
    tap_range(g, 0, p.x, xs, xe);
    tap_range(g, 1, p.y, ys, ye);
    tap_range(g, 2, p.z, zs, ze);
    xs = max(xs, x0); xe = min(xe, x0 + B - 1);
    ys = max(ys, y0); ye = min(ye, y0 + B - 1);
    zs = max(zs, z0); ze = min(ze, z0 + B - 1);
    if (c >= C) continue;
    float2 v = y[(int64_t)s * C + c];
    // temp = data * kw; temp *= taper  (src/gridFFT.cpp:1039-1108)
    const float tp = stap[s];
    v = make_float2(__fmul_rn(__fmul_rn(v.x, p.w), tp), __fmul_rn(__fmul_rn(v.y, p.w), tp));
    float wx[6];
#pragma unroll
    for (int a = 0; a < 6; a++) wx[a] = (xs + a <= xe) ? tap_w(g.lut[0], g.gmod[0], p.x, xs + a) : 0.0f;
    for (int lz = zs; lz <= ze; lz++) {
      const float wz = tap_w(g.lut[2], g.gmod[2], p.z, lz);
      for (int ly = ys; ly <= ye; ly++) {
        const float wzy = wz * tap_w(g.lut[1], g.gmod[1], p.y, ly);
        float *row = tile + ((((lz - z0) * B + (ly - y0)) * B + (xs - x0)) * 2 * G) + lane;
#pragma unroll
        for (int a = 0; a < 6; a++) {
          if (xs + a <= xe) {
            const float w = wzy * wx[a];
            atomicAdd(row + a * 2 * G, w * v.x);
            atomicAdd(row + a * 2 * G + G, w * v.y);
          }
        }
      }
    }
  }
  __syncthreads();

  const bool split = it.w != 0;
  for (int e = threadIdx.x; e < B3 * G; e += blockDim.x) {
    const int l = e % G, pt = e / G;
    const int cc = cb + l;
    if (cc >= C) continue;
    const int px = pt % B, py = (pt / B) % B, pz = pt / (B * B);
    const int64_t gi = ((((int64_t)(z0 + pz)) * g.S[1] + (y0 + py)) * g.S[0] + (x0 + px)) * C + cc;
    const float re = tile[pt * 2 * G + l], im = tile[pt * 2 * G + G + l];
    if (split) {
      atomicAdd(&grid[gi].x, re);
      atomicAdd(&grid[gi].y, im);
    } else {
      grid[gi] = make_float2(re, im);
    }
  }
}

static int grid_group(int C) {
  int G = 1;
  while (G < C && G < 16) G *= 2;
  return G;
}

mrg_status launch_grid(const GridConst &gc, const FrameTraj &ft, const float2 *y, float2 *grid, cudaStream_t st) {
  const int G = grid_group(gc.C);
  const int nchunks = (gc.C + G - 1) / G;
  if (ft.nsplit > 0) {
    const int64_t n = (int64_t)ft.nsplit * gc.B * gc.B * gc.B * gc.C;
    k_zero_tiles<<<grid_blocks(n, 256), 256, 0, st>>>(gc, ft.split_tiles, ft.nsplit, grid);
    MRG_LAUNCHED();
  }
  const size_t smem = (size_t)gc.B * gc.B * gc.B * 2 * G * sizeof(float);
  const dim3 blocks(ft.nitems, nchunks);
  void (*fn)(const GridConst, const int4 *, const int *, const float4 *, const float *, const float2 *, float2 *);
  switch (G) {
    case 1: fn = k_grid<1>; break;
    case 2: fn = k_grid<2>; break;
    case 4: fn = k_grid<4>; break;
    case 8: fn = k_grid<8>; break;
    default: fn = k_grid<16>; break;
  }
  static int attr_set[5] = {0, 0, 0, 0, 0};  // smem cap for the largest tile (16^3), once per kernel
  const int slot = G == 1 ? 0 : G == 2 ? 1 : G == 4 ? 2 : G == 8 ? 3 : 4;
  if (!attr_set[slot]) {
    MRG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::min<size_t>(16 * 16 * 16 * 2 * G * sizeof(float), 227 * 1024)));
    attr_set[slot] = 1;
  }
  if (smem > 227 * 1024) {
    set_error("gridding tile too large for shared memory");
    return MRG_ERR_INVALID;
  }
  fn<<<blocks, 256, smem, st>>>(gc, ft.items, ft.pairs, ft.spos, ft.stap, y, grid);
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// sample reordering between the user's per-coil layout and [sorted][coil]
// ---------------------------------------------------------------------------
__global__ void k_gather_samples(int nvalid, int C, const int *__restrict__ perm, const float2 *__restrict__ src,
                                 int64_t stride, float2 *__restrict__ dst) {
  const int64_t n = (int64_t)nvalid * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / C;
    const int c = (int)(e - s * C);
    dst[e] = src[(int64_t)c * stride + perm[s]];
  }
}

__global__ void k_scatter_samples(int64_t M, int nvalid, int C, const int *__restrict__ perm,
                                  const float2 *__restrict__ src, float2 *__restrict__ dst, int64_t stride) {
  const int64_t n = M * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / C;
    const int c = (int)(e - s * C);
    const float2 v = (s < nvalid) ? src[e] : make_float2(0.f, 0.f);
    dst[(int64_t)c * stride + perm[s]] = v;
  }
}

mrg_status launch_gather_samples(const FrameTraj &ft, int C, const float2 *src, int64_t stride, float2 *dst,
                                 cudaStream_t st) {
  if (ft.nvalid == 0) return MRG_OK;
  k_gather_samples<<<grid_blocks((int64_t)ft.nvalid * C, 256), 256, 0, st>>>(ft.nvalid, C, ft.perm, src, stride, dst);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status launch_scatter_samples(const FrameTraj &ft, int C, const float2 *src, float2 *dst, int64_t stride,
                                  cudaStream_t st) {
  k_scatter_samples<<<grid_blocks(ft.M * C, 256), 256, 0, st>>>(ft.M, ft.nvalid, C, ft.perm, src, dst, stride);
  MRG_LAUNCHED();
  return MRG_OK;
}

}  // namespace mrg
