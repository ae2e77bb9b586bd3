// Gridding (gridFFT::chop_grid_forward, src/gridFFT.cpp:1009-1164) on the fifth-generation
// tensor cores: tcgen05.mma with the accumulator in tensor memory.
//
// The grid is cut into regions of 8x4x4 = 128 points, one TMEM lane (one thread of the
// 128-thread CTA) per point.  For a region, the scatter of its (sample, region) pairs is
// the GEMM
//   grid[128 points][N] += W[128 points][K pairs] * V[K pairs][N],   N = 2 * coils,
// W the tap weights (wz*wy)*wx of each point for each sample, V the weighted sample
// values with real and imaginary parts as separate columns.  Both operands are split
// x = hi + lo (hi = tf32(x), lo = tf32(x - hi)) and the product taken as
// Wl*Vh + Wh*Vl + Wh*Vh in TF32, products exact to about 2^-21.
//
// Per chunk of 32 pairs the CTA stages the pairs' tap weights and values with cp.async,
// writes W and V (hi and lo) into shared memory in the K-major, unswizzled canonical
// layout, and one thread issues 12 MMAs (4 k-steps x 3 terms) into one of two TMEM
// accumulator slots, committing them to that slot's mbarrier.  While they run, the
// threads build the next chunk in the other buffer.  Each chunk is summed by the tensor
// core from zero and added into the thread's FP32 registers with round-to-nearest when
// its slot is reused: the tensor core rounds its sums toward zero, which along one long
// accumulation became a bias (measured on the mma.sync kernel: 3.4e-5 from FP64 at 256^3).
//
// Every mbarrier wait is bounded (about two seconds of SM clock); a kernel that runs
// out of time sets an error flag, waits once more (bounded) for its own MMAs, frees its
// tensor memory and returns.
#include "mrg_internal.h"

namespace mrg {

namespace {

__device__ int g_umma_error = 0;

constexpr int UK = 32;  // pairs per chunk: four k-steps of 8 TF32 values

template <int CC>
struct UmmaLayout {
  static constexpr int N = 2 * CC;              // accumulator columns
  static constexpr int A = 128 * UK * 4;        // bytes of one W operand (hi or lo)
  static constexpr int B = N * UK * 4;          // bytes of one V operand (hi or lo)
  static constexpr int BUF = 2 * A + 2 * B;     // W hi, W lo, V hi, V lo
  static constexpr int SV = UK * N * 4;         // staged sample values [k][N]
  static constexpr int SW = UK * 24 * 4;        // staged tap weights [k][24]
  static constexpr int ST = UK * 16;            // staged first taps [k]
  static constexpr int SYZ = UK * 16 * 4;       // (wz*wy) per pair and (py, pz) [k][pz*4 + py]
  static constexpr int SX = UK * 8 * 4;         // wx per pair and px [k][px]
  static constexpr int TOTAL = 2 * BUF + SV + SW + ST + SYZ + SX;
  static constexpr int TCOLS = (2 * N < 32) ? 32 : 2 * N;  // two accumulator slots
};

__device__ __forceinline__ uint32_t s_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ucp16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s_u32(dst)), "l"(src));
}
__device__ __forceinline__ void ucp8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s_u32(dst)), "l"(src));
}

// Byte offset of element (row r, k) in the K-major canonical layout without swizzle:
// 8-row x 16-byte core matrices, K-adjacent cores 128 bytes apart (LBO), 8-row groups
// 1024 bytes apart (SBO).
__device__ __forceinline__ int canon(int r, int k) { return (r >> 3) * 1024 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4; }

// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte units,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// Instruction descriptor: D F32, A and B TF32, both K-major, N >> 3, M >> 4 (M = 128).
template <int N>
__device__ __forceinline__ uint32_t idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ uint32_t tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split4(const float (&v)[4], uint4 &hi, uint4 &lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    h[i] = tf32_rn(v[i]);
    l[i] = tf32_rn(v[i] - __uint_as_float(h[i]));
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

// Bounded wait for phase `parity` of an mbarrier; false after ~2 s of SM clock.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > 4000000000LL) return false;
  }
}

// Drains accumulator slot `slot` (this thread's lane = row) into acc with
// round-to-nearest adds.
template <int N>
__device__ __forceinline__ void drain(uint32_t tmem, int slot, int warp, float (&acc)[N]) {
#pragma unroll
  for (int c0 = 0; c0 < N; c0 += 16) {
    uint32_t v[16];
    const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(slot * N + c0);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(ta));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) acc[c0 + j] = __fadd_rn(acc[c0 + j], __uint_as_float(v[j]));
  }
}

// CC coils per pass (blockIdx.y picks the chunk of coils), persistent over work items.
template <int CC, bool VEC>
__global__ void __launch_bounds__(128, 2)
    k_grid_umma(const GridConst g, BlockShape rs, int nitems, const int4 *__restrict__ items,
                const int *__restrict__ pairs, const float4 *__restrict__ swt, const int4 *__restrict__ sst,
                const float2 *__restrict__ yw, float2 *__restrict__ grid) {
  typedef UmmaLayout<CC> L;
  constexpr int N = L::N;
  constexpr int NCH = N / 4;        // 16-byte pieces per sample record
  constexpr int RPI = 128 / NCH;    // records per staging round
  extern __shared__ __align__(1024) unsigned char usm[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tslot;
  float *sv = reinterpret_cast<float *>(usm + 2 * L::BUF);
  float *sw = reinterpret_cast<float *>(usm + 2 * L::BUF + L::SV);
  int4 *stt = reinterpret_cast<int4 *>(usm + 2 * L::BUF + L::SV + L::SW);
  float *syz = reinterpret_cast<float *>(usm + 2 * L::BUF + L::SV + L::SW + L::ST);
  float *sx = reinterpret_cast<float *>(usm + 2 * L::BUF + L::SV + L::SW + L::ST + L::SYZ);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int px = tid & 7, py = (tid >> 3) & 3, pz = tid >> 5;  // this thread's point (TMEM lane = tid)
  const int C = g.C, c0 = blockIdx.y * CC, nc = min(CC, C - c0);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_u32(&tslot)),
                 "r"(L::TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_u32(&bar[0])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_u32(&bar[1])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};
  bool ok = true;

  for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
    const int4 it = __ldg(items + item);
    const int rx = it.x % rs.nb[0], ry = (it.x / rs.nb[0]) % rs.nb[1], rz = it.x / (rs.nb[0] * rs.nb[1]);
    const int x0 = rx * RGN_X, y0 = ry * RGN_Y, z0 = rz * RGN_Z;
    float acc[N];
#pragma unroll
    for (int j = 0; j < N; j++) acc[j] = 0.f;
    int buf = 0;
    for (int q0 = it.y; q0 < it.z && ok; q0 += UK, buf ^= 1) {
      const int nq = min(UK, it.z - q0);
      // ---- stage the chunk's pairs: first taps, tap weights, sample values ----
      const int s_own = (tid < nq) ? __ldg(pairs + q0 + tid) : 0;  // thread k: sample of pair k
      __shared__ int ssmp[UK];
      if (tid < UK) ssmp[tid] = s_own;
      __syncthreads();
      if (tid < nq) ucp16(stt + tid, sst + s_own);
      for (int e = tid; e < UK * 6; e += 128) {  // 6 pieces of 16 bytes per record
        const int k = e / 6, piece = e % 6;
        if (k < nq) ucp16(sw + k * 24 + 4 * piece, swt + 6 * (int64_t)ssmp[k] + piece);
      }
#pragma unroll
      for (int r0 = 0; r0 < UK; r0 += RPI) {
        const int k = r0 + tid / NCH, q = tid % NCH;  // piece q = floats 4q..4q+3 = coils 2q, 2q+1
        if (k < UK) {
          float *dst = sv + k * N + 4 * q;
          if (k < nq) {
            const float2 *v = yw + (int64_t)ssmp[k] * C + c0;
            if (VEC) {
              if (2 * q < nc) ucp16(dst, v + 2 * q);
              else *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
              if (2 * q < nc) ucp8(dst, v + 2 * q);
              else *reinterpret_cast<float2 *>(dst) = make_float2(0.f, 0.f);
              if (2 * q + 1 < nc) ucp8(dst + 2, v + 2 * q + 1);
              else *reinterpret_cast<float2 *>(dst + 2) = make_float2(0.f, 0.f);
            }
          } else {
            *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
      }
      asm volatile("cp.async.commit_group;\n" ::);
      asm volatile("cp.async.wait_group 0;\n" ::);
      __syncthreads();
      // ---- per pair: (wz*wy) for the region's 4 y and 4 z planes, wx for its 8 x ----
      {
        const int k = tid >> 2, zz = tid & 3;  // 32 pairs x 4 z planes
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 xv = make_float2(0.f, 0.f);
        if (k < nq) {
          const int4 t = stt[k];
          const float *w = sw + k * 24;
          const int az = z0 + zz - t.z;
          const float wz = (az >= 0 && az < 8) ? w[16 + az] : 0.0f;
          float wy[4];
#pragma unroll
          for (int yy = 0; yy < 4; yy++) {
            const int ay = y0 + yy - t.y;
            wy[yy] = (ay >= 0 && ay < 8) ? w[8 + ay] : 0.0f;
          }
          // (wz * wy) first, as src/gridFFT.cpp:1113-1140 multiplies them
          v = make_float4(__fmul_rn(wz, wy[0]), __fmul_rn(wz, wy[1]), __fmul_rn(wz, wy[2]), __fmul_rn(wz, wy[3]));
          const int ax0 = x0 + 2 * zz - t.x, ax1 = ax0 + 1;  // this thread also fills wx for x = 2zz, 2zz+1
          xv = make_float2((ax0 >= 0 && ax0 < 8) ? w[ax0] : 0.0f, (ax1 >= 0 && ax1 < 8) ? w[ax1] : 0.0f);
        }
        *reinterpret_cast<float4 *>(syz + k * 16 + zz * 4) = v;
        *reinterpret_cast<float2 *>(sx + k * 8 + 2 * zz) = xv;
      }
      __syncthreads();
      // ---- the slot of this buffer is free once its chunk (two back) is summed ----
      if (pending[buf]) {
        // every thread waits (bounded); they give up together so the barriers stay matched
        ok = __syncthreads_and(mbar_wait(s_u32(&bar[buf]), phase[buf]) ? 1 : 0) != 0;
        if (!ok) break;
        phase[buf] ^= 1u;
        pending[buf] = false;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        drain<N>(tmem, buf, warp, acc);
      }
      // ---- W (this thread's row) and V into buffer buf, hi and lo ----
      unsigned char *base = usm + buf * L::BUF;
      unsigned char *ah = base, *al = base + L::A, *bh = base + 2 * L::A, *bl = base + 2 * L::A + L::B;
#pragma unroll
      for (int k4 = 0; k4 < UK / 4; k4++) {
        float w4[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int k = 4 * k4 + i;
          w4[i] = __fmul_rn(syz[k * 16 + pz * 4 + py], sx[k * 8 + px]);  // (wz*wy)*wx
        }
        uint4 h, l;
        split4(w4, h, l);
        *reinterpret_cast<uint4 *>(ah + canon(tid, 4 * k4)) = h;
        *reinterpret_cast<uint4 *>(al + canon(tid, 4 * k4)) = l;
      }
#pragma unroll
      for (int u = tid; u < N * (UK / 4); u += 128) {
        const int n = u % N, k4 = u / N;
        float v4[4];
#pragma unroll
        for (int i = 0; i < 4; i++) v4[i] = sv[(4 * k4 + i) * N + n];
        uint4 h, l;
        split4(v4, h, l);
        *reinterpret_cast<uint4 *>(bh + canon(n, 4 * k4)) = h;
        *reinterpret_cast<uint4 *>(bl + canon(n, 4 * k4)) = l;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t id = idesc<N>();
        const uint32_t d = tmem + (uint32_t)(buf * N);
        const uint32_t a_h = s_u32(ah), a_l = s_u32(al), b_h = s_u32(bh), b_l = s_u32(bl);
#pragma unroll
        for (int ks = 0; ks < UK / 8; ks++) {
          const uint32_t o = (uint32_t)(ks * 256);  // 8 k = two cores along K
          mma_tf32(d, sdesc(a_l + o), sdesc(b_h + o), id, ks > 0 ? 1u : 0u);  // small terms first
          mma_tf32(d, sdesc(a_h + o), sdesc(b_l + o), id, 1u);
          mma_tf32(d, sdesc(a_h + o), sdesc(b_h + o), id, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         s_u32(&bar[buf]))
                     : "memory");
      }
      pending[buf] = true;
    }
    // ---- sum what is still in flight, then write the region ----
    for (int b = 0; b < 2 && ok; b++) {
      if (!pending[b]) continue;
      ok = __syncthreads_and(mbar_wait(s_u32(&bar[b]), phase[b]) ? 1 : 0) != 0;
      if (!ok) break;
      phase[b] ^= 1u;
      pending[b] = false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      drain<N>(tmem, b, warp, acc);
    }
    if (!ok) break;
    const int64_t gi = (((int64_t)(z0 + pz) * g.S[1] + (y0 + py)) * g.S[0] + (x0 + px)) * C + c0;
    if (it.w) {
#pragma unroll
      for (int j = 0; j < N; j++)
        if ((j >> 1) < nc) atomicAdd(reinterpret_cast<float *>(grid + gi) + j, acc[j]);
    } else if (VEC) {
      float4 *o4 = reinterpret_cast<float4 *>(grid + gi);
#pragma unroll
      for (int j = 0; j < N / 4; j++)
        if (2 * j < nc) o4[j] = make_float4(acc[4 * j], acc[4 * j + 1], acc[4 * j + 2], acc[4 * j + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < N / 2; j++)
        if (j < nc) grid[gi + j] = make_float2(acc[2 * j], acc[2 * j + 1]);
    }
    __syncthreads();  // the staging area and barriers are reused by the next item
  }
  if (!ok) {
    atomicExch(&g_umma_error, 1);
    for (int b = 0; b < 2; b++)  // let MMAs still in flight finish before the memory is freed
      if (pending[b]) mbar_wait(s_u32(&bar[b]), phase[b]);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::TCOLS));
}

}  // namespace

bool umma_supported(int C) { return C >= 8; }
int umma_default_cc(int C) { return C > 16 ? 32 : (C > 8 ? 16 : 8); }

int umma_error_flag() {
  int h = 0;
  if (cudaMemcpyFromSymbol(&h, g_umma_error, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return h;
}

template <int CC>
static mrg_status launch_umma_cc(const GridConst &gc, const FrameTraj &ft, const float2 *yw, float2 *grid,
                                 cudaStream_t st) {
  typedef UmmaLayout<CC> L;
  const bool vec = (gc.C % 2 == 0) && (((uintptr_t)yw & 15) == 0) && (((uintptr_t)grid & 15) == 0);
  static int ctas_per_sm = 0;
  if (ctas_per_sm == 0) {
    MRG_CUDA(cudaFuncSetAttribute(k_grid_umma<CC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::TOTAL));
    MRG_CUDA(cudaFuncSetAttribute(k_grid_umma<CC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::TOTAL));
    int n = 0;
    MRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_grid_umma<CC, true>, 128, L::TOTAL));
    // TMEM: at most 512 columns per SM are shared by the resident CTAs
    ctas_per_sm = std::max(1, std::min(n, 512 / L::TCOLS));
  }
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int nx = std::max(1, std::min(ft.regions.nitems, sms * ctas_per_sm));
  const dim3 blocks((unsigned)nx, (unsigned)((gc.C + CC - 1) / CC));
  const BlockShape rs = region_shape(gc);
  if (vec)
    k_grid_umma<CC, true><<<blocks, 128, L::TOTAL, st>>>(gc, rs, ft.regions.nitems, ft.regions.items,
                                                         ft.regions.pairs, ft.swt, ft.sst, yw, grid);
  else
    k_grid_umma<CC, false><<<blocks, 128, L::TOTAL, st>>>(gc, rs, ft.regions.nitems, ft.regions.items,
                                                          ft.regions.pairs, ft.swt, ft.sst, yw, grid);
  MRG_LAUNCHED();
  return MRG_OK;
}

// The caller zeroes the split regions (ft.regions.split) first.
mrg_status launch_grid_umma(const GridConst &gc, const FrameTraj &ft, int cc, const float2 *yw, float2 *grid,
                            cudaStream_t st) {
  if (!umma_supported(gc.C) || ft.regions.items == nullptr) {
    set_error("tensor-memory gridding needs >= 8 coils and region pair lists");
    return MRG_ERR_UNSUPPORTED;
  }
  if (ft.regions.nitems == 0) return MRG_OK;
  switch (cc) {
    case 8: return launch_umma_cc<8>(gc, ft, yw, grid, st);
    case 16: return launch_umma_cc<16>(gc, ft, yw, grid, st);
    default: return launch_umma_cc<32>(gc, ft, yw, grid, st);
  }
}

}  // namespace mrg
