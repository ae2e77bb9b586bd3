// One-sided Jacobi SVD of a small block matrix held in shared memory, in FP32 (FP64
// arithmetic is slow on this part).  Shared by the coil low-rank (clear.cu) and the time
// low-rank (llr.cu) kernels, whose block matrices are R x C with R the block's rows
// (voxels, times frames for the coil blocks) and C <= 32 columns (coils or frames).
//
// Rotations are applied to column pairs until every pair is orthogonal to 4e-7 relative
// (round-robin rounds; warp w rotates pairs w, w + nwarp, ... of a round), accumulating
// W: on return A W has orthogonal columns, so A = (A W) W^H with the singular values the
// column norms of A W and the right singular vectors the columns of W.  Measured against
// FP64: <= 2e-6 per threshold application up to 16 columns.
#pragma once

#include <cuda_runtime.h>

namespace mrg {

constexpr int JAC_LDV = 33;  // row pitch (float2) of W in shared memory

// Called by every thread of the CTA (blockDim a multiple of 32, C <= 32).  As: R x C
// row-major with row pitch ld >= C (As[r * ld + c]; an odd pitch spreads a warp's column
// reads over the banks); Vf: C x JAC_LDV, set to W; sg: C floats, set to the column norms
// of A W.  s_off / s_fl: two shared scalars for the CTA's reductions.
__device__ inline void jacobi_onesided_f32(float2 *As, int R, int C, int ld, float2 *Vf, float *sg, unsigned *s_off,
                                           float *s_fl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int Ce = C + (C & 1), half = Ce / 2;
  for (int e = threadIdx.x; e < C * JAC_LDV; e += blockDim.x)
    Vf[e] = make_float2((e / JAC_LDV) == (e % JAC_LDV) ? 1.f : 0.f, 0.f);
  if (warp == 0) {  // floor of the pair test: (1e-6 x the largest column norm)^2
    float mx = 0.f;
    for (int j = 0; j < C; j++) {
      float sq = 0.f;
      for (int r = lane; r < R; r += 32) {
        const float2 x = As[r * ld + j];
        sq += x.x * x.x + x.y * x.y;
      }
      for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
      mx = fmaxf(mx, sq);
    }
    if (lane == 0) *s_fl = 1e-12f * mx;
  }
  __syncthreads();
  const float fl = *s_fl;
  for (int sweep = 0; sweep < 40; sweep++) {
    if (threadIdx.x == 0) *s_off = 0u;
    __syncthreads();
    for (int rnd = 0; rnd < Ce - 1; rnd++) {
      for (int pp = warp; pp < half; pp += nwarp) {
        const int jp = pp == 0 ? 0 : 1 + (pp - 1 + rnd) % (Ce - 1);
        const int jq = 1 + (Ce - 2 - pp + rnd) % (Ce - 1);  // position Ce - 1 - pp >= 1
        if (jp >= C || jq >= C) continue;                    // the padding column of an odd C
        float al = 0.f, be = 0.f, gr = 0.f, gi = 0.f;
        for (int r = lane; r < R; r += 32) {
          const float2 x = As[r * ld + jp], y = As[r * ld + jq];
          al += x.x * x.x + x.y * x.y;
          be += y.x * y.x + y.y * y.y;
          gr += x.x * y.x + x.y * y.y;  // conj(x) y
          gi += x.x * y.y - x.y * y.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, o);
          be += __shfl_xor_sync(0xffffffffu, be, o);
          gr += __shfl_xor_sync(0xffffffffu, gr, o);
          gi += __shfl_xor_sync(0xffffffffu, gi, o);
        }
        const float ag = sqrtf(gr * gr + gi * gi);
        if (!(al > 0.f && be > 0.f && ag > 0.f)) continue;
        const float rel = ag / sqrtf(fmaxf(al, fl) * fmaxf(be, fl));
        if (lane == 0) atomicMax(s_off, __float_as_uint(rel));
        if (rel < 4e-7f) continue;
        const float zeta = (be - al) / (2.f * ag);
        const float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
        const float cs = 1.f / sqrtf(1.f + t * t), sn = cs * t;
        const float phx = gr / ag, phy = gi / ag;
        auto rot = [&](float2 *px, float2 *py) {  // x' = cs x - sn y', y' = (sn x + cs y') ph, y' = y conj(ph)
          const float2 x = *px, y0 = *py;
          const float2 y = make_float2(y0.x * phx + y0.y * phy, y0.y * phx - y0.x * phy);
          *px = make_float2(cs * x.x - sn * y.x, cs * x.y - sn * y.y);
          const float2 u = make_float2(sn * x.x + cs * y.x, sn * x.y + cs * y.y);
          *py = make_float2(u.x * phx - u.y * phy, u.x * phy + u.y * phx);
        };
        for (int r = lane; r < R; r += 32) rot(As + r * ld + jp, As + r * ld + jq);
        if (lane < C) rot(Vf + lane * JAC_LDV + jp, Vf + lane * JAC_LDV + jq);
      }
      __syncthreads();
    }
    const float off = __uint_as_float(*s_off);
    __syncthreads();
    if (off < 4e-7f) break;
  }
  for (int j = warp; j < C; j += nwarp) {  // s_j = |column j of A W|
    float sq = 0.f;
    for (int r = lane; r < R; r += 32) {
      const float2 x = As[r * ld + j];
      sq += x.x * x.x + x.y * x.y;
    }
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (lane == 0) sg[j] = sqrtf(sq);
  }
  __syncthreads();
}

}  // namespace mrg
