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
// Samples are sorted by the grid tile (B^3 points) that holds their centre, and
// their tap weights (LUT interpolation and chop sign) are computed once per
// trajectory and reused by every E and E^H call.
// Ungridding walks samples in that order (tile-local gathers hit L1/L2).
// Gridding is output-driven: a warp owns an 8x2x2 block of grid points (lane =
// point) and keeps all coils of its point in registers while it walks the list
// of samples whose kernel support touches the block (8x2x2 points: a 5-tap
// support meets 13.5 blocks on average, the fewest for 32 points); each grid value is written
// to HBM once with plain stores, without atomics.  Only blocks whose list is
// split across several work items (the dense k-space centre) add with global
// atomics into a block zeroed beforehand.
#include <algorithm>
#include <climits>
#include <functional>

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
                            float *kr_out, int *key, int *cnt, int ntiles) {
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
    // kr = kx*kx + ky*ky + kz*kz accumulated in float (src/gridFFT.cpp:1096-1106); the taper
    // exp(-kr / (2 k_rad^2)) is taken in double when the samples are sorted
    float kr = 0.0f;
    kr = __fadd_rn(kr, __fmul_rn(k[0], k[0]));
    kr = __fadd_rn(kr, __fmul_rn(k[1], k[1]));
    kr = __fadd_rn(kr, __fmul_rn(k[2], k[2]));
    // tiles in Morton (Z-curve) order, so samples that are neighbours in the sorted order
    // are neighbours in k-space at every scale and a CTA's gathers share cache lines
    int kk = 0;
    for (int b = 0; b < g.mbits; b++)
      kk |= (((cell[0] >> b) & 1) << (3 * b)) | (((cell[1] >> b) & 1) << (3 * b + 1)) |
            (((cell[2] >> b) & 1) << (3 * b + 2));
    if (!ok) kk = ntiles;
    pos[i] = make_float4(dk[0], dk[1], dk[2], w);
    kr_out[i] = kr;
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

// Exclusive prefix sums of large count arrays in three passes: per chunk of SCAN_CHUNK
// counts a CTA sum, the (few) chunk sums scanned by k_scan, then each chunk scanned in
// shared memory and offset.  out[n] = the total.  Counts are non-negative and their total
// fits in an int (pair and sample counts of one frame).
constexpr int SCAN_CHUNK = 8192;  // 1024 threads x 8 counts

__global__ void __launch_bounds__(1024) k_scan_sums(const int *__restrict__ in, int n, int *__restrict__ sums) {
  __shared__ int ws[32];
  const int base = blockIdx.x * SCAN_CHUNK;
  int s = 0;
  for (int k = threadIdx.x; k < SCAN_CHUNK; k += 1024)
    if (base + k < n) s += in[base + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = ws[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = v;
  }
}

__global__ void __launch_bounds__(1024) k_scan_chunks(const int *__restrict__ in, int n,
                                                      const int *__restrict__ offs, int *__restrict__ out) {
  __shared__ int ws[32];
  const int base = blockIdx.x * SCAN_CHUNK, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // thread t takes counts base + 8t .. base + 8t + 7
  int v[8], s = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int k = base + 8 * threadIdx.x + i;
    v[i] = k < n ? in[k] : 0;
    s += v[i];
  }
  int inc = s;  // inclusive scan of the thread sums within the warp
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int w = ws[lane], wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    ws[lane] = wi - w;  // exclusive over warps
  }
  __syncthreads();
  int run = offs[blockIdx.x] + ws[warp] + inc - s;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int k = base + 8 * threadIdx.x + i;
    if (k < n) out[k] = run;
    run += v[i];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 1023) out[n] = run;
}

// out[0..n] = exclusive prefix sums of in[0..n) and the total (out has n + 1 entries; one
// more, out[n + 1], may be written as scratch by the single-CTA path for small n).
static mrg_status launch_scan(const int *in, int *out, int n, cudaStream_t st) {
  if (n <= 4 * SCAN_CHUNK) {
    k_scan<<<1, 1024, 0, st>>>(in, out, n);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? MRG_OK : MRG_ERR_CUDA;
  }
  const int nch = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  int *sums = nullptr;
  MRG_CUDA(cudaMallocAsync(&sums, sizeof(int) * (size_t)(2 * nch + 2), st));
  int *offs = sums + nch + 1;
  k_scan_sums<<<nch, 1024, 0, st>>>(in, n, sums);
  k_scan<<<1, 1024, 0, st>>>(sums, offs, nch);
  k_scan_chunks<<<nch, 1024, 0, st>>>(in, n, offs, out);
  count_launch(3);
  const bool ok = cudaGetLastError() == cudaSuccess;
  cudaFreeAsync(sums, st);
  return ok ? MRG_OK : MRG_ERR_CUDA;
}

__device__ __forceinline__ float taper(float kr, float k_rad) {
  return (float)exp(-(double)kr / (2.0 * (double)k_rad * (double)k_rad));
}

__global__ void k_traj_sort(int64_t M, float k_rad, const int *__restrict__ key, const int *__restrict__ off, int *cur,
                            const float4 *__restrict__ pos, const float *__restrict__ kr, float4 *spos, float *stap,
                            float *skr, int *perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = key[i];
    const int s = off[k] + atomicAdd(&cur[k], 1);
    spos[s] = pos[i];
    skr[s] = kr[i];
    stap[s] = taper(kr[i], k_rad);
    perm[s] = (int)i;
  }
}

__global__ void k_count_taps(int nvalid, const int4 *__restrict__ sst, unsigned long long *total) {
  unsigned long long n = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nvalid; i += (int64_t)gridDim.x * blockDim.x) {
    const int w = sst[i].w;
    n += (unsigned long long)((w & 15) * ((w >> 4) & 15) * ((w >> 8) & 15));
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(total, n);
}

// Taps over all valid samples of a frame (sum of nx*ny*nz): the gather count of one ungrid.
mrg_status count_taps(const FrameTraj &ft, int64_t *out) {
  *out = 0;
  if (ft.nvalid == 0) return MRG_OK;
  unsigned long long *d = nullptr, h = 0;
  MRG_CUDA(cudaMalloc(&d, sizeof(h)));
  cudaMemset(d, 0, sizeof(h));
  k_count_taps<<<grid_blocks(ft.nvalid, 256), 256>>>(ft.nvalid, ft.sst, d);
  const cudaError_t e1 = cudaGetLastError();
  const cudaError_t e2 = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    set_error("tap count failed");
    return MRG_ERR_CUDA;
  }
  count_launch();
  *out = (int64_t)h;
  return MRG_OK;
}

__global__ void k_retaper(int64_t M, float k_rad, const float *__restrict__ skr, float *stap) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x)
    stap[i] = taper(skr[i], k_rad);
}

// Taper of every sample for a new k_rad (the public gridFFT::k_rad field the
// coil-map estimate lowers to the map resolution, recon_lib.cpp:2738, :2786).
mrg_status launch_retaper(const GridConst &gc, FrameTraj &ft, cudaStream_t st) {
  if (ft.M == 0) return MRG_OK;
  k_retaper<<<grid_blocks(ft.M, 256), 256, 0, st>>>(ft.M, gc.k_rad, ft.skr, ft.stap);
  MRG_LAUNCHED();
  return MRG_OK;
}

// Analytic Kaiser-Bessel kernel with the table's beta and scale:
//   K(d) = n I0(beta sqrt(1-u^2)) / I0(beta),  u = d / dwin  (d in grid units)
//   K'(d) = -n beta^2 u (I1(z)/z) / (I0(beta) dwin),  z = beta sqrt(1-u^2)
__device__ __forceinline__ double kb_value(const GridConst &g, int d, double dist) {
  const double u = dist / (double)g.dwin[d];
  if (u > 1.0) return 0.0;
  const double b = (double)g.beta[d];
  return g.kb_norm[d] * cyl_bessel_i0(b * sqrt(fmax(1.0 - u * u, 0.0))) / cyl_bessel_i0(b);
}
__device__ __forceinline__ double kb_deriv(const GridConst &g, int d, double dist) {
  const double u = dist / (double)g.dwin[d];
  if (u > 1.0) return 0.0;
  const double b = (double)g.beta[d];
  const double z = b * sqrt(fmax(1.0 - u * u, 0.0));
  const double i1z = (z > 1e-6) ? cyl_bessel_i1(z) / z : 0.5 + z * z / 16.0;
  return -g.kb_norm[d] * b * b * u * i1z / (cyl_bessel_i0(b) * (double)g.dwin[d]);
}

// Tap weights of every valid sample, computed once (src/gridFFT.cpp:1110-1148).
__global__ void k_sample_weights(GridConst g, int nvalid, const float4 *__restrict__ spos, float4 *swt, int4 *sst) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nvalid; s += gridDim.x * blockDim.x) {
    const float4 p = spos[s];
    const float dk[3] = {p.x, p.y, p.z};
    float w[24];
    int st[3], n[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      int a, b;
      tap_range(g, d, dk[d], a, b);
      st[d] = a;
      n[d] = b - a + 1;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        float v = 0.0f;
        if (k < n[d]) {
          const int l = a + k;
          if (g.eval == 1) {
            const double kv = kb_value(g, d, fabs((double)dk[d] - (double)l));
            v = (float)((l & 1) ? kv : -kv);
          } else {
            v = tap_w(g.lut[d], g.gmod[d], dk[d], l);
          }
        }
        w[8 * d + k] = v;
      }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) swt[6 * (int64_t)s + k] = make_float4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    sst[s] = make_int4(st[0], st[1], st[2], n[0] | (n[1] << 4) | (n[2] << 8));
  }
}

// (sample, block) pairs for blocks of bs.b[0] x b[1] x b[2] points: count (FILL = false)
// or fill the per-block lists.
template <bool FILL>
__global__ void k_pairs(BlockShape bs, int nvalid, const int4 *__restrict__ sst, int *pcnt, const int *__restrict__ poff,
                        int *pcur, int *pairs) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nvalid; s += gridDim.x * blockDim.x) {
    const int4 t = sst[s];
    const int nx = t.w & 15, ny = (t.w >> 4) & 15, nz = (t.w >> 8) & 15;
    const int x0 = t.x / bs.b[0], x1 = (t.x + nx - 1) / bs.b[0];
    const int y0 = t.y / bs.b[1], y1 = (t.y + ny - 1) / bs.b[1];
    const int z0 = t.z / bs.b[2], z1 = (t.z + nz - 1) / bs.b[2];
    for (int bz = z0; bz <= z1; bz++)
      for (int by = y0; by <= y1; by++)
        for (int bx = x0; bx <= x1; bx++) {
          const int blk = (bz * bs.nb[1] + by) * bs.nb[0] + bx;
          if (FILL) pairs[poff[blk] + atomicAdd(&pcur[blk], 1)] = s;
          else atomicAdd(&pcnt[blk], 1);
        }
  }
}

__global__ void k_item_count(int nblocks, const int *__restrict__ pcnt, int maxp, int *icnt) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nblocks; t += gridDim.x * blockDim.x)
    icnt[t] = max(1, (pcnt[t] + maxp - 1) / maxp);
}

__global__ void k_item_fill(int nblocks, const int *__restrict__ pcnt, const int *__restrict__ poff,
                            const int *__restrict__ icnt, const int *__restrict__ ioff, int maxp, int4 *items,
                            int *split, int *nsplit) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nblocks; t += gridDim.x * blockDim.x) {
    const int n = icnt[t];
    for (int k = 0; k < n; k++) {
      const int p0 = poff[t] + k * maxp;
      const int p1 = min(poff[t] + pcnt[t], p0 + maxp);
      items[ioff[t] + k] = make_int4(t, p0, p1, n > 1 ? 1 : 0);
    }
    if (n > 1) split[atomicAdd(nsplit, 1)] = t;
  }
}


void traj_free(FrameTraj &ft) {
  SetupScratch &x = ft.scr;
  for (void *q : {(void *)x.pos, (void *)x.tap, (void *)x.key, (void *)x.cnt, (void *)x.off, (void *)x.cur,
                  (void *)x.pcnt, (void *)x.poff, (void *)x.pcur, (void *)x.icnt, (void *)x.ioff, (void *)x.nsplit})
    cudaFree(q);
  cudaFree(ft.spos);
  cudaFree(ft.stap);
  cudaFree(ft.skr);
  cudaFree(ft.perm);
  cudaFree(ft.swt);
  cudaFree(ft.sst);
  pair_set_free(ft.blocks);
  pair_set_free(ft.regions);
  cudaFree(ft.rtab);
  cudaFree(ft.rchunk);
  cudaFree(ft.dsorted);
  cudaFree(ft.sdw);
  ft = FrameTraj();
}

// Clears a frame for a new trajectory, keeping its device arrays for reuse.
static void traj_reset(FrameTraj &ft) {
  ft.M = 0;
  ft.nvalid = 0;
  ft.has_data = false;
  ft.sdw_valid = false;
  for (PairSet *ps : {&ft.blocks, &ft.regions}) {
    ps->npairs = 0;
    ps->nitems = 0;
    ps->nsplit = 0;
    ps->built = false;
  }
  ft.nrchunks = 0;
  ft.ungrid_G = ft.ungrid_spb = ft.ungrid_cpl = ft.ungrid_uy = ft.grid_cc = 0;
  ft.tune_ungrid_ms = ft.tune_grid_ms = 0.f;
}

static mrg_status read_int(const int *dev, int *host, cudaStream_t st, const char *what) {
  if (cudaMemcpyAsync(host, dev, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    set_error(std::string(what) + ": " + cudaGetErrorString(cudaGetLastError()));
    return MRG_ERR_CUDA;
  }
  return MRG_OK;
}

mrg_status build_region_tables(FrameTraj &ft, cudaStream_t st) {
  ft.nrchunks = 0;
  const int n = ft.regions.nitems;
  if (n == 0) return MRG_OK;
  int *cnt = nullptr;
  MRG_TRY(grow(ft.scr.icnt, ft.scr.cap_icnt, n + 1));  // the item scratch is free again here
  cnt = ft.scr.icnt;
  MRG_TRY(grow(ft.rchunk, ft.cap_rchunk, n + 2));
  MRG_TRY(launch_item_chunks(ft, cnt, st));
  MRG_TRY(launch_scan(cnt, ft.rchunk, n, st));
  int total = 0;
  MRG_TRY(read_int(ft.rchunk + n, &total, st, "region chunk count failed"));
  ft.nrchunks = total;
  const int64_t nf = (int64_t)total * umma_table_floats();
  MRG_TRY(grow(ft.rtab, ft.cap_rtab, nf));
  // zero: the pad entries of a last, partial k-step must be finite (their samples are zero)
  MRG_TRY(launch_zero(ft.rtab, sizeof(float) * (size_t)std::max<int64_t>(nf, 1), st));
  return launch_region_tables(ft, st);
}

BlockShape block_shape(const GridConst &gc) {
  BlockShape bs;
  bs.b[0] = BLK_X; bs.b[1] = BLK_Y; bs.b[2] = BLK_Z;
  for (int d = 0; d < 3; d++) bs.nb[d] = gc.S[d] / bs.b[d];
  return bs;
}
BlockShape region_shape(const GridConst &gc) {
  BlockShape bs;
  bs.b[0] = RGN_X; bs.b[1] = RGN_Y; bs.b[2] = RGN_Z;
  for (int d = 0; d < 3; d++) bs.nb[d] = gc.S[d] / bs.b[d];
  return bs;
}

void pair_set_free(PairSet &ps) {
  cudaFree(ps.pairs);
  cudaFree(ps.items);
  cudaFree(ps.split);
  ps = PairSet();
}

// Pair lists of one block shape: every valid sample is listed under each block its
// support touches; each block becomes ceil(pairs / max_pairs) work items (at least one,
// so that every grid point is written), flagged when there are several (those flush
// with atomics into a pre-zeroed block).
static mrg_status build_pairs(const BlockShape &bs, int nvalid, const int4 *sst, int max_pairs, cudaStream_t st,
                              PairSet &ps, SetupScratch &x) {
  ps.npairs = 0;
  ps.nitems = 0;
  ps.nsplit = 0;
  ps.built = false;
  const int nblocks = bs.nb[0] * bs.nb[1] * bs.nb[2];
  mrg_status rs = MRG_OK;
#define PAIRS_TRY(x)         \
  do {                       \
    rs = (x);                \
    if (rs != MRG_OK) {      \
      pair_set_free(ps);     \
      return rs;             \
    }                        \
  } while (0)
#define PAIRS_LAUNCHED()                                                    \
  do {                                                                      \
    count_launch();                                                         \
    if (cudaGetLastError() != cudaSuccess) PAIRS_TRY(MRG_ERR_CUDA);         \
  } while (0)
  PAIRS_TRY(grow(x.pcnt, x.cap_pcnt, nblocks + 1));
  PAIRS_TRY(grow(x.poff, x.cap_poff, nblocks + 2));
  PAIRS_TRY(grow(x.pcur, x.cap_pcur, nblocks + 1));
  int *pcnt = x.pcnt, *poff = x.poff, *pcur = x.pcur;
  PAIRS_TRY(launch_zero(pcnt, sizeof(int) * (nblocks + 1), st));
  PAIRS_TRY(launch_zero(pcur, sizeof(int) * (nblocks + 1), st));
  if (nvalid > 0) {
    k_pairs<false><<<grid_blocks(nvalid, 256), 256, 0, st>>>(bs, nvalid, sst, pcnt, nullptr, nullptr, nullptr);
    PAIRS_LAUNCHED();
  }
  PAIRS_TRY(launch_scan(pcnt, poff, nblocks, st));
  int npairs = 0;
  PAIRS_TRY(read_int(poff + nblocks, &npairs, st, "pair count failed"));
  ps.npairs = npairs;
  PAIRS_TRY(grow(ps.pairs, ps.cap_pairs, npairs));
  if (nvalid > 0) {
    k_pairs<true><<<grid_blocks(nvalid, 256), 256, 0, st>>>(bs, nvalid, sst, nullptr, poff, pcur, ps.pairs);
    PAIRS_LAUNCHED();
  }
  PAIRS_TRY(grow(x.icnt, x.cap_icnt, nblocks + 1));
  PAIRS_TRY(grow(x.ioff, x.cap_ioff, nblocks + 2));
  PAIRS_TRY(grow(x.nsplit, x.cap_nsplit, 1));
  int *icnt = x.icnt, *ioff = x.ioff, *nsplit = x.nsplit;
  PAIRS_TRY(launch_zero(nsplit, sizeof(int), st));
  k_item_count<<<grid_blocks(nblocks, 256), 256, 0, st>>>(nblocks, pcnt, max_pairs, icnt);
  PAIRS_LAUNCHED();
  PAIRS_TRY(launch_scan(icnt, ioff, nblocks, st));
  int nitems = 0;
  PAIRS_TRY(read_int(ioff + nblocks, &nitems, st, "item count failed"));
  ps.nitems = nitems;
  PAIRS_TRY(grow(ps.items, ps.cap_items, nitems));
  PAIRS_TRY(grow(ps.split, ps.cap_split, nblocks));
  k_item_fill<<<grid_blocks(nblocks, 256), 256, 0, st>>>(nblocks, pcnt, poff, icnt, ioff, max_pairs, ps.items,
                                                         ps.split, nsplit);
  PAIRS_LAUNCHED();
  int ns = 0;
  PAIRS_TRY(read_int(nsplit, &ns, st, "item fill failed"));
  ps.nsplit = ns;
  ps.built = true;
#undef PAIRS_TRY
#undef PAIRS_LAUNCHED
  return MRG_OK;
}

mrg_status build_block_pairs(const GridConst &gc, FrameTraj &ft, int max_pairs, cudaStream_t st) {
  if (ft.blocks.built) return MRG_OK;
  return build_pairs(block_shape(gc), ft.nvalid, ft.sst, max_pairs, st, ft.blocks, ft.scr);
}

mrg_status traj_setup(const GridConst &gc, FrameTraj &ft, const float *kx, const float *ky, const float *kz,
                      const float *kw, int64_t M, int max_pairs, bool regions, cudaStream_t st) {
  traj_reset(ft);
  if (M <= 0 || M >= (int64_t)1 << 31) {
    set_error("trajectory length must be in [1, 2^31)");
    return MRG_ERR_INVALID;
  }
  const int ntiles = 1 << (3 * gc.mbits);  // Morton key space of the sort tiles
  ft.M = M;
  SetupScratch &x = ft.scr;
  mrg_status rs = MRG_OK;
#define SETUP_TRY(x)         \
  do {                       \
    rs = (x);                \
    if (rs != MRG_OK) {      \
      traj_free(ft);         \
      return rs;             \
    }                        \
  } while (0)
#define SETUP_LAUNCHED()                                                                  \
  do {                                                                                    \
    count_launch();                                                                       \
    if (cudaGetLastError() != cudaSuccess) SETUP_TRY(MRG_ERR_CUDA);                       \
  } while (0)
  // 1. positions, validity, sort key (tile of the sample centre); counting sort by tile
  SETUP_TRY(grow(x.pos, x.cap_pos, M));
  SETUP_TRY(grow(x.tap, x.cap_tap, M));
  SETUP_TRY(grow(x.key, x.cap_key, M));
  SETUP_TRY(grow(x.cnt, x.cap_cnt, ntiles + 1));
  SETUP_TRY(grow(x.off, x.cap_off, ntiles + 2));
  SETUP_TRY(grow(x.cur, x.cap_cur, ntiles + 1));
  SETUP_TRY(grow(ft.spos, ft.cap_spos, M));
  SETUP_TRY(grow(ft.stap, ft.cap_stap, M));
  SETUP_TRY(grow(ft.skr, ft.cap_skr, M));
  SETUP_TRY(grow(ft.perm, ft.cap_perm, M));
  float4 *pos = x.pos;
  float *tap = x.tap;
  int *key = x.key, *cnt = x.cnt, *off = x.off, *cur = x.cur;
  SETUP_TRY(launch_zero(cnt, sizeof(int) * (ntiles + 1), st));
  SETUP_TRY(launch_zero(cur, sizeof(int) * (ntiles + 1), st));
  k_traj_prep<<<grid_blocks(M, 256), 256, 0, st>>>(gc, kx, ky, kz, kw, M, pos, tap, key, cnt, ntiles);
  SETUP_LAUNCHED();
  SETUP_TRY(launch_scan(cnt, off, ntiles + 1, st));
  k_traj_sort<<<grid_blocks(M, 256), 256, 0, st>>>(M, gc.k_rad, key, off, cur, pos, tap, ft.spos, ft.stap, ft.skr,
                                                    ft.perm);
  SETUP_LAUNCHED();
  int nvalid = 0;
  SETUP_TRY(read_int(off + ntiles, &nvalid, st, "trajectory sort failed"));
  ft.nvalid = nvalid;

  // 2. tap weights once per trajectory
  SETUP_TRY(grow(ft.swt, ft.cap_swt, 6 * (int64_t)nvalid));
  SETUP_TRY(grow(ft.sst, ft.cap_sst, nvalid));
  k_sample_weights<<<grid_blocks(nvalid, 256), 256, 0, st>>>(gc, nvalid, ft.spos, ft.swt, ft.sst);
  SETUP_LAUNCHED();

  // 3-4. (sample, region) pair lists, work items and chunk tables for the 8x4x4 regions of
  // the tensor-memory gridding kernel when it may run; the 8x2x2 block lists of the other
  // gridding kernels are built by build_block_pairs when one of those may run
  if (regions && umma_grid_fits(gc.S)) {
    SETUP_TRY(build_pairs(region_shape(gc), nvalid, ft.sst, max_pairs, st, ft.regions, x));
    SETUP_TRY(pack_region_items(gc, ft.regions, st));
    SETUP_TRY(build_region_tables(ft, st));
  }
#undef SETUP_TRY
#undef SETUP_LAUNCHED
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// ungridding: y[s][c] = sum_taps w * grid[tap][c]  (- diff[s][c]) [* kw * taper]
// ---------------------------------------------------------------------------
// G lanes per sample, CPL coils per lane: the coil chunk [blockIdx.y*G*CPL, +G*CPL).
// A CTA walks SPB consecutive (tile-sorted) samples for one coil chunk, so the grid
// neighbourhood it reads is small enough for L1 to catch the reuse between
// neighbouring samples.  The sum is taken separably, x taps first:
//   y = sum_z wz sum_y wy sum_x wx g,
// which needs one multiply-add per tap and coil instead of forming every 3D weight.
template <int CPL>
struct UngridVec;
template <>
struct UngridVec<1> {
  typedef float2 T;
  static __device__ __forceinline__ T zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ T load(const float2 *p) { return __ldg(p); }
  static __device__ __forceinline__ void fma(float *ar, float w, T v) {
    ar[0] += w * v.x;
    ar[1] += w * v.y;
  }
};
template <>
struct UngridVec<2> {
  typedef float4 T;
  static __device__ __forceinline__ T zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  static __device__ __forceinline__ T load(const float2 *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
  static __device__ __forceinline__ void fma(float *ar, float w, T v) {
    ar[0] += w * v.x;
    ar[1] += w * v.y;
    ar[2] += w * v.z;
    ar[3] += w * v.w;
  }
};
// four coils per lane: one 32-byte load (address 32-byte aligned: C % 4 == 0)
struct F8 {
  float v[8];
};
template <>
struct UngridVec<4> {
  typedef F8 T;
  static __device__ __forceinline__ T zero() {
    F8 z;
#pragma unroll
    for (int i = 0; i < 8; i++) z.v[i] = 0.f;
    return z;
  }
  static __device__ __forceinline__ T load(const float2 *p) {
    F8 r;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]), "=f"(r.v[4]), "=f"(r.v[5]), "=f"(r.v[6]),
          "=f"(r.v[7])
        : "l"(p));
    return r;
  }
  static __device__ __forceinline__ void fma(float *ar, float w, const T &v) {
#pragma unroll
    for (int i = 0; i < 8; i++) ar[i] += w * v.v[i];
  }
};

// A window of 5 x 5 x 5 taps (every sample but those at exact half-integer positions or
// clipped at the grid's edge) is summed fully unrolled, with its weights in registers and
// every gather unpredicated, so the loads of later rows can be issued early (the kernel
// is bound by the latency of these L1 gathers).  Other windows take the general loop,
// where UY rows of taps are loaded before any of them is summed and taps beyond a
// sample's counts load zero and carry zero weights (the tables are padded).  CT: the coil
// count as a compile-time constant (0: from the plan), which turns the tap offsets into
// immediates.
template <int G, int CPL, int UY, int CT = 0>
__global__ void __launch_bounds__(256) k_ungrid(const GridConst g, int nvalid, int spb, const float4 *__restrict__ swt,
                                               const int4 *__restrict__ sst, const float4 *__restrict__ spos,
                                               const float *__restrict__ stap, const float2 *__restrict__ grid,
                                               const float2 *__restrict__ diff, float2 *__restrict__ y, int weigh) {
  typedef UngridVec<CPL> V;
  typedef typename V::T VT;
  constexpr int GPB = 256 / G;  // sample groups per CTA
  const int lane = threadIdx.x % G, grp = threadIdx.x / G;
  const int C = CT ? CT : g.C;
  const int c = (blockIdx.y * G + lane) * CPL;  // first coil of this lane
  const int64_t ys = (int64_t)g.S[0] * C, zs = (int64_t)g.S[1] * ys;
  const int64_t s_begin = (int64_t)blockIdx.x * spb;
  const int64_t s_end = min((int64_t)nvalid, s_begin + spb);
  for (int64_t gid = s_begin + grp; gid < s_end; gid += GPB) {
    const int4 t = __ldg(sst + gid);
    const int nx = t.w & 15, ny = (t.w >> 4) & 15, nz = (t.w >> 8) & 15;
    const float *w = reinterpret_cast<const float *>(swt + 6 * gid);
    const float4 wa = __ldg(swt + 6 * gid), wb = __ldg(swt + 6 * gid + 1);
    const float wx[6] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y};
    if (c >= C) continue;
    float acc[2 * CPL];
#pragma unroll
    for (int k = 0; k < 2 * CPL; k++) acc[k] = 0.f;
    const float2 *base = grid + ((int64_t)t.z * g.S[1] + t.y) * ys + (int64_t)t.x * C + c;
    if (nx == 5 && ny == 5 && nz == 5) {
      const float4 wc = __ldg(swt + 6 * gid + 2), wd = __ldg(swt + 6 * gid + 4), we = __ldg(swt + 6 * gid + 5);
      const float wy[5] = {wc.x, wc.y, wc.z, wc.w, __ldg(w + 12)};
      const float wz[5] = {wd.x, wd.y, wd.z, wd.w, we.x};
#pragma unroll
      for (int kz = 0; kz < 5; kz++) {
        float az[2 * CPL];
#pragma unroll
        for (int k = 0; k < 2 * CPL; k++) az[k] = 0.f;
#pragma unroll
        for (int ky = 0; ky < 5; ky++) {
          const float2 *row = base + kz * zs + ky * ys;
          VT v[5];
#pragma unroll
          for (int a = 0; a < 5; a++) v[a] = V::load(row + a * C);
          float ar[2 * CPL];
#pragma unroll
          for (int k = 0; k < 2 * CPL; k++) ar[k] = 0.f;
#pragma unroll
          for (int a = 0; a < 5; a++) V::fma(ar, wx[a], v[a]);
#pragma unroll
          for (int k = 0; k < 2 * CPL; k++) az[k] += wy[ky] * ar[k];
        }
#pragma unroll
        for (int k = 0; k < 2 * CPL; k++) acc[k] += wz[kz] * az[k];
      }
    } else {
    for (int kz = 0; kz < nz; kz++) {
      float az[2 * CPL];
#pragma unroll
      for (int k = 0; k < 2 * CPL; k++) az[k] = 0.f;
      for (int ky0 = 0; ky0 < ny; ky0 += UY) {
        VT v[UY][6];
#pragma unroll
        for (int u = 0; u < UY; u++) {
          const float2 *row = base + kz * zs + (ky0 + u) * ys;
#pragma unroll
          for (int a = 0; a < 6; a++)
            v[u][a] = (ky0 + u < ny && a < nx) ? V::load(row + (int64_t)a * C) : V::zero();
        }
#pragma unroll
        for (int u = 0; u < UY; u++) {
          float ar[2 * CPL];
#pragma unroll
          for (int k = 0; k < 2 * CPL; k++) ar[k] = 0.f;
#pragma unroll
          for (int a = 0; a < 6; a++) V::fma(ar, wx[a], v[u][a]);
          const float wyv = (ky0 + u < ny) ? __ldg(w + 8 + ky0 + u) : 0.f;
#pragma unroll
          for (int k = 0; k < 2 * CPL; k++) az[k] += wyv * ar[k];
        }
      }
      const float wzv = __ldg(w + 16 + kz);
#pragma unroll
      for (int k = 0; k < 2 * CPL; k++) acc[k] += wzv * az[k];
    }
    }
    float kw = 0.f, tp = 0.f;
    if (weigh) {
      kw = __ldg(&spos[gid].w);
      tp = __ldg(stap + gid);
    }
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      if (c + q >= C) break;
      const int64_t o = gid * C + c + q;
      float2 r = make_float2(acc[2 * q], acc[2 * q + 1]);
      if (diff) {
        const float2 d = diff[o];
        r.x -= d.x;
        r.y -= d.y;
      }
      if (weigh)  // temp = data * kw; temp *= taper  (src/gridFFT.cpp:1039-1108)
        r = make_float2(__fmul_rn(__fmul_rn(r.x, kw), tp), __fmul_rn(__fmul_rn(r.y, kw), tp));
      y[o] = r;
    }
  }
}

static int ungrid_group_default(int C) {
  int G = 1;
  while (G < C && G < 8) G *= 2;
  return G;
}

static mrg_status launch_ungrid_mma(int NT, const GridConst &gc, const FrameTraj &ft, const float2 *grid,
                                    const float2 *diff, float2 *y, bool weigh, cudaStream_t st);

mrg_status launch_ungrid(const GridConst &gc, const FrameTraj &ft, const float2 *grid, const float2 *diff, float2 *y,
                         bool weigh, cudaStream_t st) {
  if (ft.nvalid == 0) return MRG_OK;
  // tensor-core kernel: ungrid_G = -(n-tiles per pass); needs its alignments, else the default shape
  if (ft.ungrid_G < 0) {
    const int NT = -ft.ungrid_G;
    if (gc.C % (4 * NT) == 0 && ((uintptr_t)grid & 31) == 0 && ((uintptr_t)y & 15) == 0 && ((uintptr_t)diff & 15) == 0)
      return launch_ungrid_mma(NT, gc, ft, grid, diff, y, weigh, st);
  }
  int G = ft.ungrid_G > 0 ? ft.ungrid_G : ungrid_group_default(gc.C);
  // two coils per lane (16-byte loads) when the coil count is even and the buffers allow it,
  // four (32-byte loads) when it is a multiple of 4
  int cpl = (ft.ungrid_cpl > 0) ? ft.ungrid_cpl : ((gc.C % 2 == 0) ? 2 : 1);
  if (cpl == 4 && (gc.C % 4 != 0 || ((uintptr_t)grid & 31) != 0 || G < 4 || G > 16)) cpl = 2;
  if (cpl == 2 && (gc.C % 2 != 0 || ((uintptr_t)grid & 15) != 0)) cpl = 1;
  const int spb = ft.ungrid_spb > 0 ? ft.ungrid_spb : 256;
  const int uy = ft.ungrid_uy > 0 ? ft.ungrid_uy : 1;
  const int chunk = G * cpl;
  const dim3 blocks((unsigned)((ft.nvalid + spb - 1) / spb), (unsigned)((gc.C + chunk - 1) / chunk));
  const int wf = weigh ? 1 : 0;
  const bool c32 = gc.C == 32 && uy == 1;  // coil count as a compile-time constant
#define UNGRID_ARGS gc, ft.nvalid, spb, ft.swt, ft.sst, ft.spos, ft.stap, grid, diff, y, wf
#define UNGRID_UY(GG, PP)                                                         \
  switch (uy) {                                                                   \
    case 2: k_ungrid<GG, PP, 2><<<blocks, 256, 0, st>>>(UNGRID_ARGS); break;      \
    case 3: k_ungrid<GG, PP, 3><<<blocks, 256, 0, st>>>(UNGRID_ARGS); break;      \
    default: k_ungrid<GG, PP, 1><<<blocks, 256, 0, st>>>(UNGRID_ARGS); break;     \
  }
#define UNGRID_CASE(GG)                                                           \
  case GG:                                                                        \
    if (cpl == 4) {                                                               \
      if (c32) k_ungrid<GG, 4, 1, 32><<<blocks, 256, 0, st>>>(UNGRID_ARGS);       \
      else k_ungrid<GG, 4, 1><<<blocks, 256, 0, st>>>(UNGRID_ARGS);               \
    } else if (cpl == 2) {                                                        \
      if (c32) k_ungrid<GG, 2, 1, 32><<<blocks, 256, 0, st>>>(UNGRID_ARGS);       \
      else { UNGRID_UY(GG, 2) }                                                   \
    } else {                                                                      \
      if (c32) k_ungrid<GG, 1, 1, 32><<<blocks, 256, 0, st>>>(UNGRID_ARGS);       \
      else { UNGRID_UY(GG, 1) }                                                   \
    }                                                                             \
    break;
  switch (G) {
    case 1:
      if (cpl == 2) k_ungrid<1, 2, 1><<<blocks, 256, 0, st>>>(UNGRID_ARGS);
      else k_ungrid<1, 1, 1><<<blocks, 256, 0, st>>>(UNGRID_ARGS);
      break;
    case 2:
      if (cpl == 2) k_ungrid<2, 2, 1><<<blocks, 256, 0, st>>>(UNGRID_ARGS);
      else k_ungrid<2, 1, 1><<<blocks, 256, 0, st>>>(UNGRID_ARGS);
      break;
    UNGRID_CASE(4)
    UNGRID_CASE(8)
    UNGRID_CASE(16)
    default:
      if (c32) {
        if (cpl == 2) k_ungrid<32, 2, 1, 32><<<blocks, 256, 0, st>>>(UNGRID_ARGS);
        else k_ungrid<32, 1, 1, 32><<<blocks, 256, 0, st>>>(UNGRID_ARGS);
      } else if (cpl == 2) { UNGRID_UY(32, 2) }
      else { UNGRID_UY(32, 1) }
      break;
  }
#undef UNGRID_CASE
#undef UNGRID_UY
#undef UNGRID_ARGS
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// gridding: a warp owns an 8x2x2 block (lane = point), coils in registers
// ---------------------------------------------------------------------------
__global__ void k_zero_blocks(const GridConst g, BlockShape bs, const int *__restrict__ blocks, int n, float2 *grid) {
  const int C = g.C;
  const int per = bs.b[0] * bs.b[1] * bs.b[2] * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n * per;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int b = blocks[e / per];
    int r = (int)(e % per);
    const int c = r % C;
    r /= C;
    const int px = r % bs.b[0], py = (r / bs.b[0]) % bs.b[1], pz = r / (bs.b[0] * bs.b[1]);
    const int bx = b % bs.nb[0], by = (b / bs.nb[0]) % bs.nb[1], bz = b / (bs.nb[0] * bs.nb[1]);
    const int64_t gi =
        (((int64_t)(bz * bs.b[2] + pz) * g.S[1] + (by * bs.b[1] + py)) * g.S[0] + (bx * bs.b[0] + px)) * C + c;
    grid[gi] = make_float2(0.f, 0.f);
  }
}

__device__ __forceinline__ void cp16(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}
__device__ __forceinline__ void cp8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}

// Shared memory per warp: 32 staged pairs x (CC coil values, 24 weights, first taps).
template <int CC>
struct GridStage {
  static constexpr int VS = CC;        // float2 per staged pair
  static constexpr int WS = 24;        // floats per staged pair
  static constexpr int V = 32 * VS;
  static constexpr int W = 32 * WS;
  static constexpr int T = 32;         // int4
  static constexpr size_t bytes = V * 8 + W * 4 + T * 16;
};

// CC coils per pass (coils [c0, c0 + CC) of this blockIdx.y); VEC: coil pairs copied as 16 bytes.
// A warp stages up to 32 pairs at a time (one lane per pair, independent async
// copies), then accumulates them from shared memory into its registers.
template <int CC, bool VEC>
__global__ void __launch_bounds__(256) k_grid(const GridConst g, int nitems, const int4 *__restrict__ items,
                                             const int *__restrict__ pairs, const float4 *__restrict__ swt,
                                             const int4 *__restrict__ sst, const float2 *__restrict__ yw,
                                             float2 *__restrict__ grid) {
  extern __shared__ __align__(16) unsigned char gsm_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * 8 + warp;
  if (item >= nitems) return;
  unsigned char *base = gsm_raw + warp * GridStage<CC>::bytes;
  float2 *sv = reinterpret_cast<float2 *>(base);
  float *sw = reinterpret_cast<float *>(base + GridStage<CC>::V * 8);
  int4 *stt = reinterpret_cast<int4 *>(base + GridStage<CC>::V * 8 + GridStage<CC>::W * 4);
  const int4 it = __ldg(items + item);
  const int C = g.C;
  const int c0 = blockIdx.y * CC;
  const int nc = min(CC, C - c0);
  const int bx = it.x % g.nb[0], by = (it.x / g.nb[0]) % g.nb[1], bz = it.x / (g.nb[0] * g.nb[1]);
  const int gx = bx * BLK_X + (lane % BLK_X), gy = by * BLK_Y + ((lane / BLK_X) % BLK_Y),
            gz = bz * BLK_Z + lane / (BLK_X * BLK_Y);
  float2 acc[CC];
#pragma unroll
  for (int c = 0; c < CC; c++) acc[c] = make_float2(0.f, 0.f);
  for (int q0 = it.y; q0 < it.z; q0 += 32) {
    const int nq = min(32, it.z - q0);
    if (lane < nq) {
      const int s = __ldg(pairs + q0 + lane);
      cp16(stt + lane, sst + s);
#pragma unroll
      for (int k = 0; k < 6; k++) cp16(sw + lane * GridStage<CC>::WS + 4 * k, swt + 6 * (int64_t)s + k);
      const float2 *v = yw + (int64_t)s * C + c0;
      if (VEC) {
#pragma unroll
        for (int c = 0; c < CC / 2; c++)
          if (2 * c < nc) cp16(sv + lane * GridStage<CC>::VS + 2 * c, v + 2 * c);
      } else {
#pragma unroll
        for (int c = 0; c < CC; c++)
          if (c < nc) cp8(sv + lane * GridStage<CC>::VS + c, v + c);
      }
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncwarp();
    for (int k = 0; k < nq; k++) {
      const int4 t = stt[k];
      const int ax = gx - t.x, ay = gy - t.y, az = gz - t.z;
      const float *w = sw + k * GridStage<CC>::WS;
      const float wx = (ax >= 0 && ax < 8) ? w[ax] : 0.0f;
      const float wy = (ay >= 0 && ay < 8) ? w[8 + ay] : 0.0f;
      const float wz = (az >= 0 && az < 8) ? w[16 + az] : 0.0f;
      const float ww = (wz * wy) * wx;  // src/gridFFT.cpp:1113-1140 order
      const float2 *v = sv + k * GridStage<CC>::VS;
      if (VEC) {
#pragma unroll
        for (int c = 0; c < CC / 2; c++) {
          const float4 u = *reinterpret_cast<const float4 *>(v + 2 * c);
          acc[2 * c].x += ww * u.x;
          acc[2 * c].y += ww * u.y;
          acc[2 * c + 1].x += ww * u.z;
          acc[2 * c + 1].y += ww * u.w;
        }
      } else {
#pragma unroll
        for (int c = 0; c < CC; c++) {
          const float2 u = v[c];
          acc[c].x += ww * u.x;
          acc[c].y += ww * u.y;
        }
      }
    }
    __syncwarp();
  }
  const int64_t gi = (((int64_t)gz * g.S[1] + gy) * g.S[0] + gx) * C + c0;
  if (it.w) {
#pragma unroll
    for (int c = 0; c < CC; c++)
      if (c < nc) {
        atomicAdd(&grid[gi + c].x, acc[c].x);
        atomicAdd(&grid[gi + c].y, acc[c].y);
      }
  } else if (VEC) {
    float4 *o4 = reinterpret_cast<float4 *>(grid + gi);
#pragma unroll
    for (int c = 0; c < CC / 2; c++)
      if (2 * c < nc) o4[c] = make_float4(acc[2 * c].x, acc[2 * c].y, acc[2 * c + 1].x, acc[2 * c + 1].y);
  } else {
#pragma unroll
    for (int c = 0; c < CC; c++)
      if (c < nc) grid[gi + c] = acc[c];
  }
}

template <int CC>
static mrg_status launch_grid_cc(const GridConst &gc, const FrameTraj &ft, const float2 *yw, float2 *grid,
                                 cudaStream_t st) {
  const bool vec = (gc.C % 2 == 0) && (CC % 2 == 0) && (((uintptr_t)yw & 15) == 0);
  const dim3 blocks((unsigned)((ft.blocks.nitems + 7) / 8), (unsigned)((gc.C + CC - 1) / CC));
  const size_t smem = 8 * GridStage<CC>::bytes;
  static DeviceOnce once;
  MRG_TRY(device_once(once, [smem]() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_grid<CC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MRG_CUDA(cudaFuncSetAttribute(k_grid<CC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return MRG_OK;
  }));
  if (vec)
    k_grid<CC, true><<<blocks, 256, smem, st>>>(gc, ft.blocks.nitems, ft.blocks.items, ft.blocks.pairs, ft.swt, ft.sst, yw, grid);
  else
    k_grid<CC, false><<<blocks, 256, smem, st>>>(gc, ft.blocks.nitems, ft.blocks.items, ft.blocks.pairs, ft.swt, ft.sst, yw, grid);
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// Gridding on the tensor cores.  For one 8x2x2 block the scatter is a product
//   grid[32 points][cols] += W[32 points][pairs] * V[pairs][cols],
// W the tap weights (wz*wy)*wx of each (point, staged sample) and V the weighted
// sample values, complex values as two real columns (cols = 2 CC).  It runs as
// mma.sync m16n8k8 in TF32 with each operand split x = hi + lo (hi = tf32(x),
// lo = tf32(x - hi)) and three products Wh Vh + Wh Vl + Wl Vh, which carries the
// products to about 2^-21 relative (FP32 has 2^-24).  Each chunk of 8 pairs is
// summed by the tensor core from zero and added to the FP32 running sum with
// round-to-nearest.
//
// Fragments (PTX ISA, mma.m16n8k8 .tf32, g = lane / 4, t = lane % 4):
//   A 16x8: a0 = A[g][t], a1 = A[g+8][t], a2 = A[g][t+4], a3 = A[g+8][t+4]
//   B 8x8:  b0 = B[t][g], b1 = B[t+4][g]
//   D 16x8: d0 = D[g][2t], d1 = D[g][2t+1], d2 = D[g+8][2t], d3 = D[g+8][2t+1]
// Rows: m-tile 0 holds points (px, py, 0) as row px + 8 py, m-tile 1 the z = 1 plane.
// Columns: n-tile j, column n stands for value index n * NT + j of the staged
// record, so a lane reads NT consecutive floats of a record for B and ends with
// the 2 NT consecutive floats [2t NT, 2t NT + 2 NT) of each of its four points:
// NT whole complex coil values, stored together.
// Staged records are 16-byte chunks XOR-swizzled by the record index (stage_swz)
// so the eight lanes of each 16-byte phase hit eight different bank groups.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}
// d = A B (accumulator input zero)
__device__ __forceinline__ void mma_tf32_z(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%10,%10,%10,%10};\n"
      : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(0.0f));
}
__device__ __forceinline__ void mma_tf32(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// XOR applied to the 16-byte chunk index of staged record k.  For 8 and 4 n-tiles
// it takes 8 distinct values over any 8 consecutive records (conflict-free staging
// writes, one record per lane) and keeps the B-fragment reads conflict-free (lanes
// (g, t) of a phase read chunk 2g / 2g+1, resp. g, of records k0 + t or k0 + 4 + t).
template <int NT>
__device__ __forceinline__ int stage_swz(int k) {
  if (NT >= 8) return (k & 1) | ((k & 2) << 1) | ((k & 4) >> 1);
  if (NT == 4) return ((k & 3) << 1) | ((k & 4) >> 2);
  if (NT == 2) return k & 2;
  return 0;
}

// One chunk of 8 staged pairs: A fragments from the pairs' x weights and y/z
// products, B fragments from the swizzled records, 3 MMAs per (m-tile, n-tile)
// into a zero-based temporary added to the accumulators with round-to-nearest.
// FULL: all 8 pairs valid (no masking of stale shared memory).
template <int NT, bool FULL>
__device__ __forceinline__ void grid_mma_chunk(int k0, int nq, int gq, int tq, int gx, const int4 *stt,
                                               const float *sw, const float4 *syz, const float *sv,
                                               float (&d)[2][NT][4]) {
  constexpr int RV = 8 * NT;
  const int kA = k0 + tq, kB = k0 + tq + 4;  // the lane's two pairs (columns t and t+4 of A)
  const bool okA = FULL || kA < nq, okB = FULL || kB < nq;
  uint32_t ah[2][4], al[2][4];
  {
    const int axA = gx - stt[kA].x, axB = gx - stt[kB].x;
    float wxA = (axA >= 0 && axA < 8) ? sw[kA * 24 + axA] : 0.0f;
    float wxB = (axB >= 0 && axB < 8) ? sw[kB * 24 + axB] : 0.0f;
    float4 yA = syz[kA], yB = syz[kB];
    if (!FULL) {
      if (!okA) { wxA = 0.f; yA = make_float4(0.f, 0.f, 0.f, 0.f); }
      if (!okB) { wxB = 0.f; yB = make_float4(0.f, 0.f, 0.f, 0.f); }
    }
    // m-tile 0: rows (py 0, pz 0) and (py 1, pz 0); m-tile 1: pz = 1
    split_tf32(__fmul_rn(yA.x, wxA), ah[0][0], al[0][0]);
    split_tf32(__fmul_rn(yA.y, wxA), ah[0][1], al[0][1]);
    split_tf32(__fmul_rn(yB.x, wxB), ah[0][2], al[0][2]);
    split_tf32(__fmul_rn(yB.y, wxB), ah[0][3], al[0][3]);
    split_tf32(__fmul_rn(yA.z, wxA), ah[1][0], al[1][0]);
    split_tf32(__fmul_rn(yA.w, wxA), ah[1][1], al[1][1]);
    split_tf32(__fmul_rn(yB.z, wxB), ah[1][2], al[1][2]);
    split_tf32(__fmul_rn(yB.w, wxB), ah[1][3], al[1][3]);
  }
  // B: NT consecutive floats [gq*NT, gq*NT + NT) of records kA and kB
  float bA[NT], bB[NT];
  {
    const int f0 = gq * NT;
    const float *rA = sv + kA * RV, *rB = sv + kB * RV;
    const int zA = stage_swz<NT>(kA), zB = stage_swz<NT>(kB);
    if (NT >= 4) {
#pragma unroll
      for (int j = 0; j < NT; j += 4) {
        const int ch = (f0 + j) >> 2;
        const float4 u = *reinterpret_cast<const float4 *>(rA + 4 * (ch ^ zA));
        const float4 w = *reinterpret_cast<const float4 *>(rB + 4 * (ch ^ zB));
        bA[j] = u.x; bA[j + 1] = u.y; bA[j + 2] = u.z; bA[j + 3] = u.w;
        bB[j] = w.x; bB[j + 1] = w.y; bB[j + 2] = w.z; bB[j + 3] = w.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < NT; j++) {
        const int f = f0 + j;
        bA[j] = rA[4 * ((f >> 2) ^ zA) + (f & 3)];
        bB[j] = rB[4 * ((f >> 2) ^ zB) + (f & 3)];
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NT; j++) {
    uint32_t bh0, bl0, bh1, bl1;
    split_tf32(okA ? bA[j] : 0.f, bh0, bl0);
    split_tf32(okB ? bB[j] : 0.f, bh1, bl1);
#pragma unroll
    for (int m = 0; m < 2; m++) {
      // the tensor core rounds its sums toward zero: take each chunk's three products
      // from zero (small terms first) and add the chunk to the running sum rounded to
      // nearest, so the truncation does not build up a bias along a long sum
      float t[4];
      mma_tf32_z(t, al[m], bh0, bh1);
      mma_tf32(t, ah[m], bl0, bl1);
      mma_tf32(t, ah[m], bh0, bh1);
#pragma unroll
      for (int e = 0; e < 4; e++) d[m][j][e] = __fadd_rn(d[m][j][e], t[e]);
    }
  }
}

template <int NT, bool VEC>
__global__ void __launch_bounds__(256, 2) k_grid_mma(const GridConst g, int nitems, const int4 *__restrict__ items,
                                                 const int *__restrict__ pairs, const float4 *__restrict__ swt,
                                                 const int4 *__restrict__ sst, const float2 *__restrict__ yw,
                                                 float2 *__restrict__ grid) {
  constexpr int CC = 4 * NT;   // coils per pass
  constexpr int RV = 2 * CC;   // floats per staged record
  constexpr int NCH = RV / 4;  // 16-byte chunks per record
  extern __shared__ __align__(16) unsigned char gsm_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * 8 + warp;
  if (item >= nitems) return;
  unsigned char *base = gsm_raw + warp * (GridStage<CC>::bytes + 32 * 16);
  float *sv = reinterpret_cast<float *>(base);
  float *sw = reinterpret_cast<float *>(base + GridStage<CC>::V * 8);
  int4 *stt = reinterpret_cast<int4 *>(base + GridStage<CC>::V * 8 + GridStage<CC>::W * 4);
  float4 *syz = reinterpret_cast<float4 *>(base + GridStage<CC>::V * 8 + GridStage<CC>::W * 4 + GridStage<CC>::T * 16);
  const int4 it = __ldg(items + item);
  const int C = g.C;
  const int c0 = blockIdx.y * CC;
  const int nc = min(CC, C - c0);
  const int bx = it.x % g.nb[0], by = (it.x / g.nb[0]) % g.nb[1], bz = it.x / (g.nb[0] * g.nb[1]);
  const int gq = lane >> 2, tq = lane & 3;
  const int gx = bx * BLK_X + gq, gy0 = by * BLK_Y, gz0 = bz * BLK_Z;
  float d[2][NT][4];
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int j = 0; j < NT; j++)
#pragma unroll
      for (int e = 0; e < 4; e++) d[m][j][e] = 0.f;

  for (int q0 = it.y; q0 < it.z; q0 += 32) {
    const int nq = min(32, it.z - q0);
    // Staging, with the lanes of a record copying neighbouring 16-byte pieces so each
    // copy instruction touches few records (one lane per scattered record would cost a
    // shared-memory wavefront per lane): lane k holds sample index s of pair k.
    const int s_own = (lane < nq) ? __ldg(pairs + q0 + lane) : 0;
    if (lane < nq) cp16(stt + lane, sst + s_own);
    // weights: 8 lanes per record (6 copy one 16-byte piece each), 4 records per round
#pragma unroll
    for (int r0 = 0; r0 < 32; r0 += 4) {
      const int rec = r0 + (lane >> 3), piece = lane & 7;
      const int s = __shfl_sync(0xffffffffu, s_own, rec);
      if (rec < nq && piece < 6) cp16(sw + rec * 24 + 4 * piece, swt + 6 * (int64_t)s + piece);
    }
    // sample values: NCH lanes per record, 32 / NCH records per round
    constexpr int RPI = 32 / NCH;
#pragma unroll
    for (int r0 = 0; r0 < 32; r0 += RPI) {
      const int rec = r0 + lane / NCH, q = lane % NCH;  // chunk q = coils 2q, 2q+1
      const int s = __shfl_sync(0xffffffffu, s_own, rec);
      if (rec < nq) {
        const float2 *v = yw + (int64_t)s * C + c0;
        float *dst = sv + rec * RV + 4 * (q ^ stage_swz<NT>(rec));
        if (VEC) {
          if (2 * q < nc) cp16(dst, v + 2 * q);
          else *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
          if (2 * q < nc) cp8(dst, v + 2 * q);
          else *reinterpret_cast<float2 *>(dst) = make_float2(0.f, 0.f);
          if (2 * q + 1 < nc) cp8(dst + 2, v + 2 * q + 1);
          else *reinterpret_cast<float2 *>(dst + 2) = make_float2(0.f, 0.f);
        }
      }
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncwarp();
    // each pair's y/z weight products for this block's two y and two z planes,
    // (wz*wy) first as src/gridFFT.cpp:1113-1140 multiplies them
    if (lane < nq) {
      const int4 tt = stt[lane];
      const float *w = sw + lane * 24;
      const int ay = gy0 - tt.y, az = gz0 - tt.z;
      const float wy0 = (ay >= 0 && ay < 8) ? w[8 + ay] : 0.0f;
      const float wy1 = (ay + 1 >= 0 && ay + 1 < 8) ? w[9 + ay] : 0.0f;
      const float wz0 = (az >= 0 && az < 8) ? w[16 + az] : 0.0f;
      const float wz1 = (az + 1 >= 0 && az + 1 < 8) ? w[17 + az] : 0.0f;
      syz[lane] = make_float4(__fmul_rn(wz0, wy0), __fmul_rn(wz0, wy1), __fmul_rn(wz1, wy0), __fmul_rn(wz1, wy1));
    }
    __syncwarp();
    for (int k0 = 0; k0 < nq; k0 += 8) {
      if (k0 + 8 <= nq) grid_mma_chunk<NT, true>(k0, nq, gq, tq, gx, stt, sw, syz, sv, d);
      else grid_mma_chunk<NT, false>(k0, nq, gq, tq, gx, stt, sw, syz, sv, d);
    }
    __syncwarp();
  }
  // the lane's points (gx, gy0 + h, gz0 + m) hold floats [2 t NT, 2 t NT + 2 NT) of the chunk
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float o[2 * NT];
#pragma unroll
      for (int j = 0; j < NT; j++) {
        o[j] = d[m][j][2 * h];
        o[NT + j] = d[m][j][2 * h + 1];
      }
      const int cl = tq * NT;  // first coil of the lane within the chunk
      const int64_t gi = (((int64_t)(gz0 + m) * g.S[1] + (gy0 + h)) * g.S[0] + gx) * C + c0 + cl;
      if (it.w) {
#pragma unroll
        for (int j = 0; j < NT; j++)
          if (cl + j < nc) {
            atomicAdd(&grid[gi + j].x, o[2 * j]);
            atomicAdd(&grid[gi + j].y, o[2 * j + 1]);
          }
      } else if (VEC && NT >= 2) {
        float4 *o4 = reinterpret_cast<float4 *>(grid + gi);
#pragma unroll
        for (int j = 0; j < NT / 2; j++)
          if (cl + 2 * j < nc) o4[j] = make_float4(o[4 * j], o[4 * j + 1], o[4 * j + 2], o[4 * j + 3]);
      } else {
#pragma unroll
        for (int j = 0; j < NT; j++)
          if (cl + j < nc) grid[gi + j] = make_float2(o[2 * j], o[2 * j + 1]);
      }
    }
}

template <int NT>
static mrg_status launch_grid_mma(const GridConst &gc, const FrameTraj &ft, const float2 *yw, float2 *grid,
                                  cudaStream_t st) {
  constexpr int CC = 4 * NT;
  const bool vec = (gc.C % 2 == 0) && (((uintptr_t)yw & 15) == 0) && (((uintptr_t)grid & 15) == 0);
  const dim3 blocks((unsigned)((ft.blocks.nitems + 7) / 8), (unsigned)((gc.C + CC - 1) / CC));
  const size_t smem = 8 * (GridStage<CC>::bytes + 32 * 16);  // + the y/z products of 32 pairs
  static DeviceOnce once;
  MRG_TRY(device_once(once, [smem]() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_grid_mma<NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MRG_CUDA(cudaFuncSetAttribute(k_grid_mma<NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return MRG_OK;
  }));
  if (vec)
    k_grid_mma<NT, true><<<blocks, 256, smem, st>>>(gc, ft.blocks.nitems, ft.blocks.items, ft.blocks.pairs, ft.swt, ft.sst, yw, grid);
  else
    k_grid_mma<NT, false><<<blocks, 256, smem, st>>>(gc, ft.blocks.nitems, ft.blocks.items, ft.blocks.pairs, ft.swt, ft.sst, yw, grid);
  MRG_LAUNCHED();
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// ungridding on the tensor cores (mma.sync m16n8k8, TF32 in three terms)
//
// A warp takes 16 consecutive samples of the sorted order (neighbours in space) and
// walks the union of their tap windows one row of 8 x-points at a time; each row is
// one k-step
//   D[16 samples][8 NT values] += W[16 samples][8 points] G[8 points][8 NT values],
// W the samples' 3D tap weights wx wy wz (zero outside a sample's window) and G the
// interleaved complex coil values of this pass's 4 NT coils at the row's 8 points.
// Every grid value is loaded once per 16 samples instead of once per sample (the
// CUDA-core kernel is bound by those L1 gathers).  Column n of n-tile j stands for
// value NT n + j of a point, so a lane loads NT consecutive floats of a point for B
// and ends with 2 NT consecutive floats (NT whole coils) of each of its two samples.
// Products are split into TF32 high and low parts (hi = x with the low 13 mantissa
// bits cleared, lo = x - hi, exact); lo's own low bits are dropped by the tensor core,
// so each product carries a relative error near 2^-21.  Each row starts its D from
// zero and is added to the FP32 accumulators with round-to-nearest adds: the tensor
// core's accumulation rounds towards zero, which over a whole window biases the sum.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void split_tf32_trunc(float x, uint32_t &hi, uint32_t &lo) {
  hi = __float_as_uint(x) & 0xffffe000u;
  lo = __float_as_uint(x - __uint_as_float(hi));
}

template <int NT>
struct UmVec {
  float v[NT];
};
template <int NT>
__device__ __forceinline__ void um_load(UmVec<NT> &r, const float *p) {
  if constexpr (NT == 8) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]), "=f"(r.v[4]), "=f"(r.v[5]), "=f"(r.v[6]),
          "=f"(r.v[7])
        : "l"(p));
  } else if constexpr (NT == 4) {
    const float4 q = __ldg(reinterpret_cast<const float4 *>(p));
    r.v[0] = q.x, r.v[1] = q.y, r.v[2] = q.z, r.v[3] = q.w;
  } else if constexpr (NT == 2) {
    const float2 q = __ldg(reinterpret_cast<const float2 *>(p));
    r.v[0] = q.x, r.v[1] = q.y;
  } else {
    r.v[0] = __ldg(p);
  }
}

// weight i of a sample's axis table (n taps; zero outside the window)
__device__ __forceinline__ float um_w(const float *w, int i, int n) { return (i >= 0 && i < n) ? __ldg(w + i) : 0.f; }

template <int NT>
__global__ void __launch_bounds__(256, 2)
    k_ungrid_mma(const GridConst g, int nvalid, int spb, const float4 *__restrict__ swt, const int4 *__restrict__ sst,
                 const float4 *__restrict__ spos, const float *__restrict__ stap, const float2 *__restrict__ grid,
                 const float2 *__restrict__ diff, float2 *__restrict__ y, int weigh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  const int C = g.C;
  const int c0 = blockIdx.y * 4 * NT;  // first coil of this pass
  const int64_t ps = 2 * (int64_t)C;   // floats per grid point
  const int64_t ys = (int64_t)g.S[0] * ps, zs = (int64_t)g.S[1] * ys;
  const float *gbase = reinterpret_cast<const float *>(grid) + 2 * c0 + NT * gq;
  const int64_t s_begin = (int64_t)blockIdx.x * spb;
  const int64_t s_end = min((int64_t)nvalid, s_begin + spb);
  for (int64_t s0 = s_begin + 16 * warp; s0 < s_end; s0 += 16 * 8) {
    // lanes l and l + 16 describe sample s0 + l; samples past the end have empty windows
    const int64_t sl = s0 + (lane & 15);
    int4 t = make_int4(0, 0, 0, 0);
    int nx = 0, ny = 0, nz = 0;
    if (sl < s_end) {
      t = __ldg(sst + sl);
      nx = t.w & 15, ny = (t.w >> 4) & 15, nz = (t.w >> 8) & 15;
    }
    const bool live = sl < s_end;
    const int x0 = __reduce_min_sync(0xffffffffu, live ? t.x : INT_MAX);
    const int x1 = __reduce_max_sync(0xffffffffu, live ? t.x + nx : INT_MIN);
    const int y0 = __reduce_min_sync(0xffffffffu, live ? t.y : INT_MAX);
    const int y1 = __reduce_max_sync(0xffffffffu, live ? t.y + ny : INT_MIN);
    const int z0 = __reduce_min_sync(0xffffffffu, live ? t.z : INT_MAX);
    const int z1 = __reduce_max_sync(0xffffffffu, live ? t.z + nz : INT_MIN);
    // this lane's two samples: rows gq and gq + 8 of the fragments
    int sx[2], sy[2], sz[2], cx[2], cy[2], cz[2];
    const float *wt[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int src = gq + 8 * h;
      sx[h] = __shfl_sync(0xffffffffu, t.x, src);
      sy[h] = __shfl_sync(0xffffffffu, t.y, src);
      sz[h] = __shfl_sync(0xffffffffu, t.z, src);
      cx[h] = __shfl_sync(0xffffffffu, nx, src);
      cy[h] = __shfl_sync(0xffffffffu, ny, src);
      cz[h] = __shfl_sync(0xffffffffu, nz, src);
      wt[h] = reinterpret_cast<const float *>(swt + 6 * (s0 + src));
    }
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int nyu = y1 - y0, nrows = nyu * (z1 - z0);
    for (int xb = x0; xb < x1; xb += 8) {
      // a0 = W[gq][tq], a1 = W[gq+8][tq], a2 = W[gq][tq+4], a3 = W[gq+8][tq+4]
      const float wx0 = um_w(wt[0], xb + tq - sx[0], cx[0]), wx1 = um_w(wt[1], xb + tq - sx[1], cx[1]);
      const float wx2 = um_w(wt[0], xb + tq + 4 - sx[0], cx[0]), wx3 = um_w(wt[1], xb + tq + 4 - sx[1], cx[1]);
      // points past the grid's edge carry zero weight: load a point that exists instead
      const int xa = min(xb + tq, g.S[0] - 1), xc = min(xb + tq + 4, g.S[0] - 1);
      const float *pa = gbase + xa * ps, *pc = gbase + xc * ps;
      UmVec<NT> ba, bc, na, nc;
      um_load<NT>(ba, pa + z0 * zs + y0 * ys);
      um_load<NT>(bc, pc + z0 * zs + y0 * ys);
      int yy = y0, zz = z0;
      for (int r = 0; r < nrows; r++) {
        // next row's values in flight while this one is multiplied
        int yn = yy + 1, zn = zz;
        if (yn == y1) yn = y0, zn++;
        if (r + 1 < nrows) {
          um_load<NT>(na, pa + zn * zs + yn * ys);
          um_load<NT>(nc, pc + zn * zs + yn * ys);
        }
        const float wyz0 = um_w(wt[0] + 16, zz - sz[0], cz[0]) * um_w(wt[0] + 8, yy - sy[0], cy[0]);
        const float wyz1 = um_w(wt[1] + 16, zz - sz[1], cz[1]) * um_w(wt[1] + 8, yy - sy[1], cy[1]);
        uint32_t ah[4], al[4];
        split_tf32_trunc(wx0 * wyz0, ah[0], al[0]);
        split_tf32_trunc(wx1 * wyz1, ah[1], al[1]);
        split_tf32_trunc(wx2 * wyz0, ah[2], al[2]);
        split_tf32_trunc(wx3 * wyz1, ah[3], al[3]);
#pragma unroll
        for (int j = 0; j < NT; j++) {
          uint32_t bh0, bl0, bh1, bl1;
          split_tf32_trunc(ba.v[j], bh0, bl0);
          split_tf32_trunc(bc.v[j], bh1, bl1);
          float d[4];
          mma_tf32_z(d, al, bh0, bh1);
          mma_tf32(d, ah, bl0, bl1);
          mma_tf32(d, ah, bh0, bh1);
#pragma unroll
          for (int i = 0; i < 4; i++) acc[j][i] = __fadd_rn(acc[j][i], d[i]);
        }
        ba = na;
        bc = nc;
        yy = yn;
        zz = zn;
      }
    }
    // lane holds values [2 NT tq, 2 NT tq + 2 NT) of rows gq and gq + 8: value m < NT is
    // column 2 tq of n-tile m, value NT + m column 2 tq + 1 of n-tile m
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int64_t s = s0 + gq + 8 * h;
      if (s >= s_end) continue;
      float kw = 0.f, tp = 0.f;
      if (weigh) {
        kw = __ldg(&spos[s].w);
        tp = __ldg(stap + s);
      }
      float v[2 * NT];
#pragma unroll
      for (int m = 0; m < NT; m++) {
        v[m] = acc[m][2 * h];
        v[NT + m] = acc[m][2 * h + 1];
      }
      const int64_t o = s * C + c0 + NT * tq;
#pragma unroll
      for (int q = 0; q < NT; q++) {
        float2 r = make_float2(v[2 * q], v[2 * q + 1]);
        if (diff) {
          const float2 dd = diff[o + q];
          r.x -= dd.x;
          r.y -= dd.y;
        }
        if (weigh)  // temp = data * kw; temp *= taper  (src/gridFFT.cpp:1039-1108)
          r = make_float2(__fmul_rn(__fmul_rn(r.x, kw), tp), __fmul_rn(__fmul_rn(r.y, kw), tp));
        v[2 * q] = r.x;
        v[2 * q + 1] = r.y;
      }
      if constexpr (NT >= 2) {
#pragma unroll
        for (int q = 0; q < NT; q += 2)
          *reinterpret_cast<float4 *>(y + o + q) = make_float4(v[2 * q], v[2 * q + 1], v[2 * q + 2], v[2 * q + 3]);
      } else {
        y[o] = make_float2(v[0], v[1]);
      }
    }
  }
}

// n-tiles per pass of the tensor-core ungridding kernel (0: not available for C coils)
int ungrid_mma_nt(int C) {
  if (C % 32 == 0) return 8;
  if (C % 16 == 0) return 4;
  if (C % 8 == 0) return 2;
  if (C % 4 == 0) return 1;
  return 0;
}

static mrg_status launch_ungrid_mma(int NT, const GridConst &gc, const FrameTraj &ft, const float2 *grid,
                                    const float2 *diff, float2 *y, bool weigh, cudaStream_t st) {
  const int spb = ft.ungrid_spb > 0 ? ft.ungrid_spb : 512;
  const dim3 blocks((unsigned)((ft.nvalid + spb - 1) / spb), (unsigned)(gc.C / (4 * NT)));
  const int wf = weigh ? 1 : 0;
#define UMMA_ARGS gc, ft.nvalid, spb, ft.swt, ft.sst, ft.spos, ft.stap, grid, diff, y, wf
  switch (NT) {
    case 8: k_ungrid_mma<8><<<blocks, 256, 0, st>>>(UMMA_ARGS); break;
    case 4: k_ungrid_mma<4><<<blocks, 256, 0, st>>>(UMMA_ARGS); break;
    case 2: k_ungrid_mma<2><<<blocks, 256, 0, st>>>(UMMA_ARGS); break;
    default: k_ungrid_mma<1><<<blocks, 256, 0, st>>>(UMMA_ARGS); break;
  }
#undef UMMA_ARGS
  MRG_LAUNCHED();
  return MRG_OK;
}

// n-tiles (4 coils each) per pass of the tensor-core kernel when none was tuned.
static int default_grid_nt(int C) { return C > 16 ? 8 : (C > 8 ? 4 : (C > 4 ? 2 : 1)); }

bool grid_cc_allowed(int C, const FrameTraj &ft, int cc) {
  if (cc >= 0) return cc == 0 || cc == 8 || cc == 16;
  if (cc > -100) return (cc == -1 || cc == -2 || cc == -4 || cc == -8) && -cc <= default_grid_nt(C);
  const int c = -cc - 100;
  return (c == 8 || c == 16 || c == 32) && umma_supported(C) && ft.regions.built && c <= umma_default_cc(C);
}

mrg_status launch_grid(const GridConst &gc, const FrameTraj &ft, const float2 *yw, float2 *grid, cudaStream_t st) {
  const int C = gc.C;
  // tcgen05 kernel over 8x4x4 regions: grid_cc = -(100 + coils per pass)
  if (ft.grid_cc <= -100 || (ft.grid_cc == 0 && gc.grid_mode == 3)) {
    if (ft.regions.nsplit > 0) {
      const BlockShape rs = region_shape(gc);
      const int64_t n = (int64_t)ft.regions.nsplit * RGN_X * RGN_Y * RGN_Z * C;
      k_zero_blocks<<<grid_blocks(n, 256), 256, 0, st>>>(gc, rs, ft.regions.split, ft.regions.nsplit, grid);
      MRG_LAUNCHED();
    }
    return launch_grid_umma(gc, ft, ft.grid_cc <= -100 ? -ft.grid_cc - 100 : umma_default_cc(C), yw, grid, st);
  }
  if (!ft.blocks.built) {
    set_error("block pair lists not built for this frame's gridding kernel");
    return MRG_ERR_STATE;
  }
  if (ft.blocks.nsplit > 0) {
    const int64_t n = (int64_t)ft.blocks.nsplit * BLK_X * BLK_Y * BLK_Z * C;
    k_zero_blocks<<<grid_blocks(n, 256), 256, 0, st>>>(gc, block_shape(gc), ft.blocks.split, ft.blocks.nsplit, grid);
    MRG_LAUNCHED();
  }
  if (ft.grid_cc < 0 || (ft.grid_cc == 0 && gc.grid_mode == 2)) {
    switch (ft.grid_cc < 0 ? -ft.grid_cc : default_grid_nt(C)) {
      case 1: return launch_grid_mma<1>(gc, ft, yw, grid, st);
      case 2: return launch_grid_mma<2>(gc, ft, yw, grid, st);
      case 4: return launch_grid_mma<4>(gc, ft, yw, grid, st);
      default: return launch_grid_mma<8>(gc, ft, yw, grid, st);
    }
  }
  if (ft.grid_cc == 16 && C > 16) return launch_grid_cc<16>(gc, ft, yw, grid, st);
  if (ft.grid_cc == 8 && C > 8) return launch_grid_cc<8>(gc, ft, yw, grid, st);
  if (C <= 1) return launch_grid_cc<1>(gc, ft, yw, grid, st);
  if (C <= 2) return launch_grid_cc<2>(gc, ft, yw, grid, st);
  if (C <= 4) return launch_grid_cc<4>(gc, ft, yw, grid, st);
  if (C <= 8) return launch_grid_cc<8>(gc, ft, yw, grid, st);
  if (C <= 16) return launch_grid_cc<16>(gc, ft, yw, grid, st);
  if (C <= 24) return launch_grid_cc<24>(gc, ft, yw, grid, st);
  return launch_grid_cc<32>(gc, ft, yw, grid, st);
}


// ---------------------------------------------------------------------------
// differentiable E: d(tap weight)/dk and the fused value + derivative gather
// ---------------------------------------------------------------------------
__global__ void k_sample_dweights(GridConst g, int nvalid, const float4 *__restrict__ spos,
                                  const int4 *__restrict__ sst, float4 *sdw) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nvalid; s += gridDim.x * blockDim.x) {
    const float4 p = spos[s];
    const int4 t = sst[s];
    const float dk[3] = {p.x, p.y, p.z};
    const int st[3] = {t.x, t.y, t.z};
    const int n[3] = {t.w & 15, (t.w >> 4) & 15, (t.w >> 8) & 15};
    float w[24];
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        float v = 0.0f;
        if (k < n[d]) {
          const int l = st[d] + k;
          const double diff = (double)dk[d] - (double)l;
          // d/dk [chop(l) K(|dk - l|)] = chop(l) K'(|d|) sign(d) * grid ratio
          double dv = kb_deriv(g, d, fabs(diff)) * (diff < 0 ? -1.0 : 1.0) * (double)g.grid[d];
          v = (float)((l & 1) ? dv : -dv);
        }
        w[8 * d + k] = v;
      }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) sdw[6 * (int64_t)s + k] = make_float4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  }
}

mrg_status launch_sample_dweights(const GridConst &gc, FrameTraj &ft, cudaStream_t st) {
  MRG_TRY(grow(ft.sdw, ft.cap_sdw, 6 * (int64_t)ft.nvalid));
  if (ft.nvalid > 0) {
    k_sample_dweights<<<grid_blocks(ft.nvalid, 256), 256, 0, st>>>(gc, ft.nvalid, ft.spos, ft.sst, ft.sdw);
    MRG_LAUNCHED();
  }
  ft.sdw_valid = true;
  return MRG_OK;
}

template <int G>
__global__ void __launch_bounds__(256) k_ungrid_grad(const GridConst g, int nvalid, int64_t M,
                                                    const float4 *__restrict__ swt, const float4 *__restrict__ sdw,
                                                    const int4 *__restrict__ sst, const int *__restrict__ perm,
                                                    const float2 *__restrict__ grid, float2 *__restrict__ ys,
                                                    float *__restrict__ gk, double *loss) {
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int lane = threadIdx.x % G;
  const bool valid = gid < nvalid;
  const int C = g.C;
  const int64_t S0 = g.S[0], S1 = g.S[1];
  float gx = 0.f, gy = 0.f, gz = 0.f;
  double ls = 0.0;
  if (valid) {
    const int4 t = __ldg(sst + gid);
    const int nx = t.w & 15, ny = (t.w >> 4) & 15, nz = (t.w >> 8) & 15;
    const float *w = reinterpret_cast<const float *>(swt + 6 * gid);
    const float *dw = reinterpret_cast<const float *>(sdw + 6 * gid);
    for (int cb = 0; cb < C; cb += G) {
      const int c = cb + lane;
      if (c >= C) break;
      float2 v = make_float2(0.f, 0.f), vx = v, vy = v, vz = v;
      for (int kz = 0; kz < nz; kz++) {
        const float wz = __ldg(w + 16 + kz), dwz = __ldg(dw + 16 + kz);
        for (int ky = 0; ky < ny; ky++) {
          const float wyv = __ldg(w + 8 + ky), dwy = __ldg(dw + 8 + ky);
          const float a = wz * wyv, bz = dwz * wyv, by = wz * dwy;
          const float2 *row = grid + (((int64_t)(t.z + kz) * S1 + (t.y + ky)) * S0 + t.x) * C + c;
          for (int kx = 0; kx < nx; kx++) {
            const float wxv = __ldg(w + kx), dwx = __ldg(dw + kx);
            const float2 gv = __ldg(row + (int64_t)kx * C);
            const float f0 = a * wxv, fx = a * dwx, fy = by * wxv, fz = bz * wxv;
            v.x += f0 * gv.x; v.y += f0 * gv.y;
            vx.x += fx * gv.x; vx.y += fx * gv.y;
            vy.x += fy * gv.x; vy.y += fy * gv.y;
            vz.x += fz * gv.x; vz.y += fz * gv.y;
          }
        }
      }
      const int64_t o = gid * C + c;
      const float2 yv = ys[o];
      const float2 r = make_float2(v.x - yv.x, v.y - yv.y);
      ys[o] = make_float2(2.f * r.x, 2.f * r.y);
      // dL/dk = sum_c 2 Re(conj(r) dv/dk)
      gx += 2.f * (r.x * vx.x + r.y * vx.y);
      gy += 2.f * (r.x * vy.x + r.y * vy.y);
      gz += 2.f * (r.x * vz.x + r.y * vz.y);
      ls += (double)r.x * r.x + (double)r.y * r.y;
    }
  }
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) {
    gx += __shfl_xor_sync(0xffffffffu, gx, off);
    gy += __shfl_xor_sync(0xffffffffu, gy, off);
    gz += __shfl_xor_sync(0xffffffffu, gz, off);
  }
  if (valid && lane == 0) {
    const int64_t u = perm[gid];
    gk[u] = gx;
    gk[M + u] = gy;
    gk[2 * M + u] = gz;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, off);
  if ((threadIdx.x & 31) == 0 && ls != 0.0) atomicAdd(loss, ls);
}

// Samples that do not contribute: E is 0 there, so r = -y and dL/dk = 0.
__global__ void k_grad_invalid(int64_t M, int nvalid, int C, const int *__restrict__ perm,
                               const float2 *__restrict__ y, int64_t stride, float *gk, double *loss) {
  double ls = 0.0;
  for (int64_t s = nvalid + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < M; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = perm[s];
    gk[u] = 0.f;
    gk[M + u] = 0.f;
    gk[2 * M + u] = 0.f;
    for (int c = 0; c < C; c++) {
      const float2 v = y[(int64_t)c * stride + u];
      ls += (double)v.x * v.x + (double)v.y * v.y;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, off);
  if ((threadIdx.x & 31) == 0 && ls != 0.0) atomicAdd(loss, ls);
}

mrg_status launch_ungrid_grad(const GridConst &gc, const FrameTraj &ft, const float2 *grid, float2 *ysorted,
                              const float2 *y_user, int64_t stride, float *grad_k, double *loss, cudaStream_t st) {
  if (ft.nvalid > 0) {
    int G = 1;
    while (G < gc.C && G < 32) G *= 2;
    const int blocks = (int)(((int64_t)ft.nvalid * G + 255) / 256);
#define GRAD_ARGS gc, ft.nvalid, ft.M, ft.swt, ft.sdw, ft.sst, ft.perm, grid, ysorted, grad_k, loss
    switch (G) {
      case 1: k_ungrid_grad<1><<<blocks, 256, 0, st>>>(GRAD_ARGS); break;
      case 2: k_ungrid_grad<2><<<blocks, 256, 0, st>>>(GRAD_ARGS); break;
      case 4: k_ungrid_grad<4><<<blocks, 256, 0, st>>>(GRAD_ARGS); break;
      case 8: k_ungrid_grad<8><<<blocks, 256, 0, st>>>(GRAD_ARGS); break;
      case 16: k_ungrid_grad<16><<<blocks, 256, 0, st>>>(GRAD_ARGS); break;
      default: k_ungrid_grad<32><<<blocks, 256, 0, st>>>(GRAD_ARGS); break;
    }
#undef GRAD_ARGS
    MRG_LAUNCHED();
  }
  if (ft.M > ft.nvalid) {
    k_grad_invalid<<<grid_blocks(ft.M - ft.nvalid, 256), 256, 0, st>>>(ft.M, ft.nvalid, gc.C, ft.perm, y_user, stride,
                                                                       grad_k, loss);
    MRG_LAUNCHED();
  }
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: times the candidate launch shapes of this frame on the plan's own
// buffers (contents irrelevant for timing) and keeps the fastest.
//   ungridding: lanes per sample (coil chunk) G and samples per CTA
//   gridding:   coils per pass CC (registers and occupancy against pair re-reads)
// ---------------------------------------------------------------------------
static float time_ms(cudaStream_t st, const std::function<mrg_status()> &f, int reps) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  if (f() != MRG_OK) {  // warm
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return 1e30f;
  }
  cudaEventRecord(a, st);
  for (int r = 0; r < reps; r++)
    if (f() != MRG_OK) break;
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

mrg_status autotune_frame(const GridConst &gc, FrameTraj &ft, float2 *grid, float2 *y, cudaStream_t st) {
  if (ft.nvalid == 0) return MRG_OK;
  float best = 1e30f;
  int bestG = ungrid_group_default(gc.C), bestS = 256, bestP = 1;
  for (int cpl : {1, 2, 4}) {
    if (gc.C % cpl) continue;
    for (int G : {4, 8, 16, 32}) {
      if (G * cpl > 2 * gc.C && G > 4) continue;
      if (cpl == 4 && G > 16) continue;
      for (int spb : {128, 512}) {
        ft.ungrid_G = G;
        ft.ungrid_spb = spb;
        ft.ungrid_cpl = cpl;
        ft.ungrid_uy = 1;
        const float ms = time_ms(st, [&]() { return launch_ungrid(gc, ft, grid, nullptr, y, false, st); }, 2);
        if (ms < best) {
          best = ms;
          bestG = G;
          bestS = spb;
          bestP = cpl;
        }
      }
    }
  }
  ft.ungrid_G = bestG;
  ft.ungrid_spb = bestS;
  ft.ungrid_cpl = bestP;
  ft.ungrid_uy = 1;
  int bestU = 1;
  if (bestG >= 4 && bestP < 4) {
    for (int uy : {2, 3}) {
      ft.ungrid_uy = uy;
      const float ms = time_ms(st, [&]() { return launch_ungrid(gc, ft, grid, nullptr, y, false, st); }, 2);
      if (ms < best) {
        best = ms;
        bestU = uy;
      }
    }
  }
  ft.ungrid_uy = bestU;
  // tensor-core kernel: wins only where samples are dense (16 consecutive samples share most
  // of their windows, e.g. 1.86 against 2.5 ms at 128^3 x 32 with every spoke inside |k| < 8);
  // for a full 3D radial trajectory it is several times slower (windows spread apart)
  if (const int nt = ungrid_mma_nt(gc.C)) {
    const int keepG = ft.ungrid_G, keepS = ft.ungrid_spb, keepP = ft.ungrid_cpl, keepU = ft.ungrid_uy;
    int mmaS = 0;
    for (int spb : {256}) {
      ft.ungrid_G = -nt;
      ft.ungrid_spb = spb;
      ft.ungrid_cpl = 1;
      ft.ungrid_uy = 1;
      const float ms = time_ms(st, [&]() { return launch_ungrid(gc, ft, grid, nullptr, y, false, st); }, 2);
      if (ms < best) {
        best = ms;
        mmaS = spb;
      }
    }
    if (mmaS) {
      ft.ungrid_spb = mmaS;
    } else {
      ft.ungrid_G = keepG, ft.ungrid_spb = keepS, ft.ungrid_cpl = keepP, ft.ungrid_uy = keepU;
    }
  }
  ft.tune_ungrid_ms = best;
  best = 1e30f;
  int bestCC = 0;
  // CUDA-core kernel: all coils, 16 or 8 per pass; mma.sync kernel (-n): 4n coils per pass;
  // tcgen05 kernel (-(100 + c)): c coils per pass
  for (int cc : {0, 16, 8, -8, -4, -2, -1, -132, -116, -108}) {
    const int mode = cc >= 0 ? 1 : (cc > -100 ? 2 : 3);
    if (gc.grid_mode != 0 && gc.grid_mode != mode) continue;
    if (mode != 3 && !ft.blocks.built) continue;
    if (mode == 1 && cc > 0 && gc.C <= cc) continue;
    if (mode == 2 && -cc > default_grid_nt(gc.C)) continue;  // more coils per pass than the plan has
    if (mode == 2 && -cc < default_grid_nt(gc.C) / 2) continue;
    if (mode == 3) {
      const int c = -cc - 100;
      if (!umma_supported(gc.C) || !ft.regions.built) continue;
      if (c > umma_default_cc(gc.C) || c < umma_default_cc(gc.C) / 2) continue;
    }
    ft.grid_cc = cc;
    float ms = time_ms(st, [&]() { return launch_grid(gc, ft, y, grid, st); }, 2);
    if (mode == 3 && read_wait_error(gc)) {  // gave up waiting for its MMAs: never pick it
      ms = 1e30f;
      MRG_CUDA(cudaMemset(gc.err, 0, sizeof(int)));
    }
    if (ms < best) {
      best = ms;
      bestCC = cc;
    }
  }
  ft.grid_cc = bestCC;
  ft.tune_grid_ms = best;
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

// ---------------------------------------------------------------------------
// sample reordering between the user's per-coil layout and [sorted][coil]
// ---------------------------------------------------------------------------
__global__ void k_gather_samples(int nvalid, int C, const int *__restrict__ perm, const float2 *__restrict__ src,
                                 int64_t stride, float2 *__restrict__ dst, const float4 *__restrict__ spos,
                                 const float *__restrict__ stap) {
  const int64_t n = (int64_t)nvalid * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / C;
    const int c = (int)(e - s * C);
    float2 v = src[(int64_t)c * stride + perm[s]];
    if (spos) {
      const float kw = spos[s].w, tp = stap[s];
      v = make_float2(__fmul_rn(__fmul_rn(v.x, kw), tp), __fmul_rn(__fmul_rn(v.y, kw), tp));
    }
    dst[e] = v;
  }
}

__global__ void k_weigh_samples(int nvalid, int C, const float2 *__restrict__ src, float2 *__restrict__ dst,
                                const float4 *__restrict__ spos, const float *__restrict__ stap) {
  const int64_t n = (int64_t)nvalid * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / C;
    const float kw = spos[s].w, tp = stap[s];
    const float2 v = src[e];
    dst[e] = make_float2(__fmul_rn(__fmul_rn(v.x, kw), tp), __fmul_rn(__fmul_rn(v.y, kw), tp));
  }
}

mrg_status launch_weigh_samples(const FrameTraj &ft, int C, const float2 *src, float2 *dst, cudaStream_t st) {
  if (ft.nvalid == 0) return MRG_OK;
  k_weigh_samples<<<grid_blocks((int64_t)ft.nvalid * C, 256), 256, 0, st>>>(ft.nvalid, C, src, dst, ft.spos, ft.stap);
  MRG_LAUNCHED();
  return MRG_OK;
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
                                 cudaStream_t st, bool weigh) {
  if (ft.nvalid == 0) return MRG_OK;
  k_gather_samples<<<grid_blocks((int64_t)ft.nvalid * C, 256), 256, 0, st>>>(
      ft.nvalid, C, ft.perm, src, stride, dst, weigh ? ft.spos : nullptr, weigh ? ft.stap : nullptr);
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
