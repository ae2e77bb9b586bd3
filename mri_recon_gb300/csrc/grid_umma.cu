// Gridding (gridFFT::chop_grid_forward, src/gridFFT.cpp:1009-1164) on the fifth-generation
// tensor cores: tcgen05.mma with the operand W and the accumulators in tensor memory.
//
// The grid is cut into regions of 8x4x4 = 128 points, one TMEM lane per point.  For a
// region, the scatter of its (sample, region) pairs is the GEMM
//   grid[128 points][N] += W[128 points][K pairs] * V[K pairs][N],   N = 2 * coils,
// W the tap weights (wz*wy)*wx of each point for each sample, V the weighted sample
// values with real and imaginary parts as separate columns.  Both operands are split
// x = hi + lo (hi = x with the low 13 mantissa bits cleared, lo = x - hi exactly; the
// tensor core drops lo's own low bits) and the product taken as Wl*Vh + Wh*Vl + Wh*Vh
// in TF32, each product within about 2^-20 of the FP32 one.
//
// One persistent CTA per SM (512 builder threads in four warpgroups, each thread owning the
// TMEM lane of one point, and one MMA warp) walks its work items chunk by chunk.  The
// trajectory set-up tabulates, per 96-pair chunk, (wz*wy) of the region's 16 (z, y) rows
// and wx of its 8 x columns for every pair (k_region_tables).  Per chunk: the chunk's table
// and its pairs' sample values are copied with cp.async one chunk ahead; each warpgroup
// writes three k-steps of W (hi and lo, its threads' own rows) into tensor memory with
// tcgen05.st, all threads write V into shared memory (K-major canonical layout), and the
// MMA warp issues up to 36 MMAs (12 k-steps x 3 terms, A read from tensor memory) into one
// of two accumulator slots, committing them to the slot's mbarrier.  While they run the CTA
// prepares the next chunk in the other slot.  The tensor core adds into its accumulator
// rounding toward zero (measured: bit-identical to an RZ emulation), so each chunk is
// summed from zero and added into the thread's FP32 registers with round-to-nearest when
// its slot is retired (two chunks later); along a whole region the truncation would
// otherwise build up a bias.  A work item is written when its last chunk is retired,
// through a shared-memory buffer so that each warp stores contiguous bytes.
//
// Every mbarrier wait is bounded (GridConst::wait_ns of the GPU's global timer, two
// seconds by default); a kernel whose wait runs out sets the plan's error word, waits
// (bounded, at least the default limit) for the MMAs it already issued, frees its tensor
// memory and returns, and the plan's next synchronising call reports MRG_ERR_TIMEOUT.
#include "mrg_internal.h"

namespace mrg {

namespace {

constexpr int TK = 96;      // pairs per chunk: twelve k-steps of 8 TF32 values
constexpr int TP = TK + 4;  // row pitch (floats) of the per-chunk weight tables: conflict-free 16-byte reads
constexpr int TROWS = 24;   // table rows: (wz*wy) of the region's 16 (z, y) rows, then wx of its 8 x
constexpr int NBLD = 512;   // builder threads: four warpgroups; warp w reaches TMEM lanes 32 (w % 4) .. + 31
constexpr int NTHR = NBLD + 32;  // and one warp that issues the MMAs

template <int CC>
struct TcLayout {
  static constexpr int N = 2 * CC;               // accumulator columns
  static constexpr int NQ = N / 4;               // accumulator columns drained by each warpgroup
  static constexpr int BOP = N * TK * 4;         // one V operand (hi or lo), K-major canonical
  static constexpr int SV = TK * N * 4;          // staged sample values [k][N]
  static constexpr int STAB = TROWS * TP * 4;    // staged chunk table [row][k]
  static constexpr int STAGE = SV + STAB;
  static constexpr int OFF_B = 0;                             // 2 slots x (V hi, V lo)
  static constexpr int OFF_STAGE = OFF_B + 4 * BOP;           // 2 staging buffers
  static constexpr int RP = N + 4;                            // row pitch (floats) of the region buffer
  static constexpr int OFF_R = OFF_STAGE + 2 * STAGE;         // a finished region [128 points][RP]
  static constexpr int USED = OFF_R + 128 * RP * 4;
  // more than half of the SM's shared memory, so one CTA per SM owns all 512 TMEM columns
  static constexpr int TOTAL = USED > 120 * 1024 ? USED : 120 * 1024;
  // tensor memory: accumulators at columns [0, 2N), W of slot s at A0 + 2 TK s (hi) and
  // A0 + 2 TK s + TK (lo)
  static constexpr int A0 = 2 * N;
  static constexpr int TCOLS = 512;
  static_assert(A0 + 4 * TK <= TCOLS, "tensor memory columns");
  static_assert(NQ % 4 == 0 && NQ >= 4, "drain width");
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
// TK * 32 bytes apart (SBO).
__device__ __forceinline__ int canon(int r, int k) {
  return (r >> 3) * (TK * 32) + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte units,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((TK * 32) >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// Instruction descriptor: D F32, A and B TF32, both K-major, N >> 3, M >> 4 (M = 128).
template <int N>
__device__ __forceinline__ uint32_t idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ uint32_t hi_bits(float x) { return __float_as_uint(x) & 0xffffe000u; }

// d (+)= A B with A (128 x 8) in tensor memory, B from a shared-memory descriptor
__device__ __forceinline__ void mma_tA(uint32_t d, uint32_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
      "r"(a), "l"(b), "r"(id), "r"(accumulate));
}

// 8 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tst8(uint32_t ta, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(ta), "r"(r[0]),
               "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
               : "memory");
}

__device__ __forceinline__ long long gtimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return (long long)t;
}

// Bounded wait for phase `parity` of an mbarrier; false once `limit_ns` of the global
// timer have passed.  try_wait itself may suspend the thread for a while before it reports
// failure, so a limit of 0 takes one non-blocking test_wait instead: it gives up at once
// unless the phase has already completed.  Between tries the thread sleeps `nap` ns, so a
// waiting warp takes few issue slots from the others.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit_ns, unsigned nap = 32) {
  if (limit_ns <= 0) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
  }
  const long long t0 = gtimer_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (gtimer_ns() - t0 >= limit_ns) return false;
    __nanosleep(nap);
  }
}

__device__ __forceinline__ void flag_wait_error(const GridConst &g) {
  if (g.err) atomicExch(g.err, MRG_WAIT_EXPIRED);
}

// Drains this warp's NQ columns of an accumulator slot (lane = row) into acc with
// round-to-nearest adds: all loads issued, one wait (tied to the loaded registers so no
// use can move above it).
template <int NQ>
__device__ __forceinline__ void drain(uint32_t ta, float (&acc)[NQ]) {
  uint32_t v[NQ];
#pragma unroll
  for (int c0 = 0; c0 < NQ; c0 += 4)
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v[c0]), "=r"(v[c0 + 1]), "=r"(v[c0 + 2]), "=r"(v[c0 + 3])
                 : "r"(ta + (uint32_t)c0));
  if constexpr (NQ == 16) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                   "+r"(v[15])::"memory");
  } else if constexpr (NQ == 8) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]),
                   "+r"(v[7])::"memory");
  } else {
    static_assert(NQ == 4, "drain width");
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3])::"memory");
  }
#pragma unroll
  for (int j = 0; j < NQ; j++) acc[j] = __fadd_rn(acc[j], __uint_as_float(v[j]));
}

// Issues the cp.async copies of one chunk into staging buffer `st`: its table (the first
// 8 ceil(nq / 8) columns of each row, from `tab`) and its sample values (pair indices
// already in shared memory, `idx`); rows k >= nq of the sample values are zeroed.
template <int CC, bool VEC>
__device__ __forceinline__ void stage_chunk(unsigned char *st, const int *idx, int nq, int tid, int C, int c0, int nc,
                                            const float *__restrict__ tab, const float2 *__restrict__ yw) {
  typedef TcLayout<CC> L;
  constexpr int N = L::N, NCH = N / 4;
  float *sv = reinterpret_cast<float *>(st);
  float *stb = reinterpret_cast<float *>(st + L::SV);
  const int pr = 2 * ((nq + 7) >> 3);  // 16-byte pieces per row
  for (int e = tid; e < TROWS * pr; e += NBLD) {
    const int row = e / pr, o = TP * row + 4 * (e - row * pr);
    ucp16(stb + o, tab + o);
  }
#pragma unroll
  for (int e0 = 0; e0 < TK * NCH; e0 += NBLD) {
    const int e = e0 + tid;
    const int k = e / NCH, q = e % NCH;  // piece q = floats 4q..4q+3 = coils 2q, 2q+1
    float *dst = sv + k * N + 4 * q;
    if (e < TK * NCH) {
      if (k < nq) {
        const float2 *v = yw + (int64_t)idx[k] * C + c0;
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
}

// Copies the pair (sample) indices of one chunk into `idx`.
__device__ __forceinline__ void stage_idx(int *idx, const int *__restrict__ pairs, int q0, int nq, int tid) {
  if (tid < nq) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s_u32(idx + tid)), "l"(pairs + q0 + tid));
}

// Region origin packed into a work item's x field, unsigned: x0 | y0 << 11 | z0 << 22
// (11, 11 and 10 bits; a z origin of 512 or more sets bit 31, so the fields are unpacked
// with unsigned shifts).
__device__ __forceinline__ int pack_origin(int x0, int y0, int z0) {
  return (int)((unsigned)x0 | ((unsigned)y0 << 11) | ((unsigned)z0 << 22));
}
__device__ __forceinline__ void unpack_origin(int packed, int &x0, int &y0, int &z0) {
  const unsigned u = (unsigned)packed;
  x0 = (int)(u & 2047u);
  y0 = (int)((u >> 11) & 2047u);
  z0 = (int)(u >> 22);
}

// Chunks of each region work item (none for an item without pairs).
__global__ void k_item_chunks(int nitems, const int4 *__restrict__ items, int *cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x) {
    const int4 it = items[i];
    cnt[i] = (it.z - it.y + TK - 1) / TK;
  }
}

// The per-chunk tables of the region work items (one CTA per item, one thread per pair):
// the products the gridding kernel multiplies into W, (wz * wy) for the region's 4 z and 4
// y planes (wz times wy first, as src/gridFFT.cpp:1113-1140) and wx for its 8 x columns,
// zero where a plane lies outside the sample's taps.  They depend on the trajectory only.
__global__ void k_region_tables(int nitems, const int4 *__restrict__ items, const int *__restrict__ pairs,
                                const int *__restrict__ rchunk, const float4 *__restrict__ swt,
                                const int4 *__restrict__ sst, float *__restrict__ rtab) {
  for (int i = blockIdx.x; i < nitems; i += gridDim.x) {
    const int4 it = items[i];
    int x0, y0, z0;
    unpack_origin(it.x, x0, y0, z0);
    const int ch0 = rchunk[i];
    for (int q = it.y + threadIdx.x; q < it.z; q += blockDim.x) {
      const int s = pairs[q];
      const int4 t = sst[s];
      float w[24];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const float4 v = swt[6 * (int64_t)s + k];
        w[4 * k] = v.x;
        w[4 * k + 1] = v.y;
        w[4 * k + 2] = v.z;
        w[4 * k + 3] = v.w;
      }
      const int r = q - it.y;
      float *o = rtab + (int64_t)(ch0 + r / TK) * (TROWS * TP) + r % TK;
#pragma unroll
      for (int zz = 0; zz < 4; zz++) {
        const int az = z0 + zz - t.z;
        const float wz = (az >= 0 && az < 8) ? w[16 + az] : 0.0f;
#pragma unroll
        for (int yy = 0; yy < 4; yy++) {
          const int ay = y0 + yy - t.y;
          o[(zz * 4 + yy) * TP] = __fmul_rn(wz, (ay >= 0 && ay < 8) ? w[8 + ay] : 0.0f);
        }
      }
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int ax = x0 + j - t.x;
        o[(16 + j) * TP] = (ax >= 0 && ax < 8) ? w[ax] : 0.0f;
      }
    }
  }
}

// Work item x field as the packed region origin.
__global__ void k_pack_regions(BlockShape rs, int nitems, int4 *items) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x) {
    const int r = items[i].x;
    const int rx = r % rs.nb[0], ry = (r / rs.nb[0]) % rs.nb[1], rz = r / (rs.nb[0] * rs.nb[1]);
    items[i].x = pack_origin(rx * RGN_X, ry * RGN_Y, rz * RGN_Z);
  }
}

// A CTA's walk over its chunks: item (-1 past the end), its work item, first pair and
// table chunk.
struct ChunkPos {
  int item, q0, ch;
  int4 it;
};
__device__ __forceinline__ ChunkPos first_chunk(int item, int nitems, const int4 *__restrict__ items,
                                                const int *__restrict__ rchunk) {
  ChunkPos p;
  p.item = item < nitems ? item : -1;
  p.it = p.item >= 0 ? __ldg(items + item) : make_int4(0, 0, 0, 0);
  p.ch = p.item >= 0 ? __ldg(rchunk + item) : 0;
  p.q0 = p.it.y;
  return p;
}
__device__ __forceinline__ ChunkPos next_chunk(const ChunkPos &p, int nitems, const int4 *__restrict__ items,
                                               const int *__restrict__ rchunk) {
  if (p.item < 0) return p;
  if (p.q0 + TK < p.it.z) {
    ChunkPos n = p;
    n.q0 += TK;
    n.ch += 1;
    return n;
  }
  return first_chunk(p.item + gridDim.x, nitems, items, rchunk);
}

__device__ __forceinline__ void bld_sync() { asm volatile("bar.sync 1, %0;" ::"n"(NBLD) : "memory"); }
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool bld_and(bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, 1, %2, q;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(NBLD)
      : "memory");
  return r != 0;
}

// CC coils per pass (blockIdx.y picks the chunk of coils), one persistent CTA per SM over
// the work items; the CTA walks its items' chunks in order (an item without pairs is one
// empty chunk).  Warps 0-15 build the operands: thread tid owns point tid % 128 (its TMEM
// lane), warpgroup g = tid / 128 writes k-steps g, g + 4, g + 8 of W and drains accumulator
// columns [g NQ, g NQ + NQ).  Warp 16 issues the MMAs.  Per slot s: full[s] (the 16
// builder warps arrive when the slot's operands are written) and done[s] (the MMAs'
// commit, or a plain arrive for an empty chunk); the builders wait done[s] of chunk c - 2
// before they reuse slot s for chunk c, so neither barrier runs two phases ahead of its
// waiter.
template <int CC, bool VEC>
__global__ void __launch_bounds__(NTHR, 1)
    k_grid_umma(const GridConst g, int nitems, const int4 *__restrict__ items, const int *__restrict__ pairs,
                const int *__restrict__ rchunk, const float *__restrict__ rtab, const float2 *__restrict__ yw,
                float2 *__restrict__ grid) {
  typedef TcLayout<CC> L;
  constexpr int N = L::N, NQ = L::NQ;
  extern __shared__ __align__(1024) unsigned char usm[];
  __shared__ __align__(8) uint64_t full[2], done[2];
  __shared__ uint32_t tslot;
  __shared__ int slot_nks[2];
  __shared__ __align__(16) int sidx[3][TK];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int C = g.C, c0 = blockIdx.y * CC, nc = min(CC, C - c0);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_u32(&tslot)),
                 "r"(L::TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < 2; s++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_u32(&full[s])), "r"(NBLD / 32));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_u32(&done[s])), "r"(1));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;

  if (warp == NBLD / 32) {
    // ---------------- MMA warp ----------------
    const uint32_t id = idesc<N>();
    for (int c = 0;; c++) {
      const int s = c & 1;
      if (!mbar_wait(s_u32(&full[s]), (uint32_t)((c >> 1) & 1), g.wait_ns, 256)) {
        flag_wait_error(g);
        break;
      }
      const int nks = slot_nks[s];
      if (nks < 0) break;  // the builders are done
      if ((tid & 31) == 0) {
        if (nks > 0) {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t d = tmem + (uint32_t)(s * N);
          const uint32_t a_h = tmem + (uint32_t)(L::A0 + 2 * TK * s), a_l = a_h + TK;
          const uint32_t bb = s_u32(usm + L::OFF_B + s * 2 * L::BOP);
          const uint64_t dh = sdesc(bb), dl = sdesc(bb + L::BOP);
#pragma unroll
          for (int ks = 0; ks < TK / 8; ks++) {
            if (ks < nks) {
              const uint64_t o = (uint64_t)(ks * 16);  // 8 k = two cores = 256 bytes
              mma_tA(d, a_l + 8 * ks, dh + o, id, ks > 0 ? 1u : 0u);  // small terms first
              mma_tA(d, a_h + 8 * ks, dl + o, id, 1u);
              mma_tA(d, a_h + 8 * ks, dh + o, id, 1u);
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           s_u32(&done[s]))
                       : "memory");
        } else {
          mbar_arrive(s_u32(&done[s]));
        }
      }
      __syncwarp();
    }
  } else {
    // ---------------- builder warps ----------------
    const int wg = tid >> 7, pt = tid & 127;
    const int px = pt & 7, py = (pt >> 3) & 3, pz = pt >> 5;  // this thread's point (TMEM lane = pt)
    const uint32_t lane_base = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    // per slot s, bit s: a chunk handed to the MMA warp and not yet summed / that chunk ends
    // its work item / the item is a split region / the done[s] phase to wait for next (bit
    // masks keep them in registers); org0, org1: the packed region origin of slot 0's and
    // slot 1's chunk
    unsigned outstanding = 0u, slast = 0u, ssplit = 0u, dphase = 0u;
    int org0 = 0, org1 = 0;
    bool ok = true;
    float acc[NQ];
#pragma unroll
    for (int j = 0; j < NQ; j++) acc[j] = 0.f;
    // A finished region goes out through shared memory so that each warp stores (or, into a
    // pre-zeroed split region, adds) contiguous bytes: the threads put their accumulators in
    // the region buffer, then thread u writes 16 bytes of point u / (N / 4).  An item without
    // pairs writes zeros (nothing for a split region).  All builder threads call it together.
    float *rbuf = reinterpret_cast<float *>(usm + L::OFF_R);
    auto write_region = [&](int packed, bool split, bool zero) {
      if (zero && split) return;
      int rx0, ry0, rz0;
      unpack_origin(packed, rx0, ry0, rz0);
      // a region outside the grid would mean a corrupt work item: report it, write nothing
      // (the condition is the same for every builder thread, so their barriers stay matched)
      if (rx0 + RGN_X > g.S[0] || ry0 + RGN_Y > g.S[1] || rz0 + RGN_Z > g.S[2]) {
        if (tid == 0 && g.err) atomicExch(g.err, MRG_REGION_RANGE);
        return;
      }
      if (!zero) {
        bld_sync();  // the previous region's readers are done with the buffer
        float4 *d = reinterpret_cast<float4 *>(rbuf + pt * L::RP + wg * NQ);
#pragma unroll
        for (int j = 0; j < NQ / 4; j++) d[j] = make_float4(acc[4 * j], acc[4 * j + 1], acc[4 * j + 2], acc[4 * j + 3]);
        bld_sync();
      }
      auto point_base = [&](int p) -> int64_t {  // grid index (float2) of coil c0 at point p
        return (((int64_t)(rz0 + (p >> 5)) * g.S[1] + (ry0 + ((p >> 3) & 3))) * g.S[0] + (rx0 + (p & 7))) * C + c0;
      };
      if (VEC) {
        constexpr int NCH = N / 4;  // 16-byte pieces per point: coils 2q, 2q + 1 in piece q
        for (int u = tid; u < 128 * NCH; u += NBLD) {
          const int p = u / NCH, q = u - p * NCH;
          if (2 * q >= nc) continue;
          float4 *o = reinterpret_cast<float4 *>(grid + point_base(p)) + q;
          const float4 v = zero ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(rbuf + p * L::RP + 4 * q);
          if (split) atomicAdd(o, v);
          else *o = v;
        }
      } else {
        for (int u = tid; u < 128 * CC; u += NBLD) {
          const int p = u / CC, q = u - p * CC;  // coil c0 + q
          if (q >= nc) continue;
          float2 *o = grid + point_base(p) + q;
          const float2 v = zero ? make_float2(0.f, 0.f) : *reinterpret_cast<const float2 *>(rbuf + p * L::RP + 2 * q);
          if (split) {
            atomicAdd(&o->x, v.x);
            atomicAdd(&o->y, v.y);
          } else {
            *o = v;
          }
        }
      }
    };
    // Waits (bounded) for the chunk last handed over in slot s and sums it; when that chunk
    // ends its item, the sum is the item's and goes out to the grid.  Chunks are summed in
    // the order they were handed over and an item is written as soon as its last chunk is
    // summed, so acc only ever holds one item.  The builders give up together so their
    // barriers stay matched.
    auto retire = [&](int s) -> bool {
      if (!((outstanding >> s) & 1u)) return true;
      if (!bld_and(mbar_wait(s_u32(&done[s]), (dphase >> s) & 1u, g.wait_ns))) return false;
      dphase ^= 1u << s;
      outstanding &= ~(1u << s);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      drain<NQ>(lane_base + (uint32_t)(s * N + wg * NQ), acc);
      if ((slast >> s) & 1u) {
        write_region(s ? org1 : org0, (ssplit >> s) & 1u, false);
#pragma unroll
        for (int j = 0; j < NQ; j++) acc[j] = 0.f;
      }
      return true;
    };
    // Chunks c, c + 1 and c + 2 are known at the top of iteration c; c + 3 is looked up there,
    // so a new work item's descriptor (a global load) has a whole iteration to arrive before
    // its pair indices are staged.
    ChunkPos cur = first_chunk(blockIdx.x, nitems, items, rchunk);
    ChunkPos nxt = next_chunk(cur, nitems, items, rchunk);
    ChunkPos nxt2 = next_chunk(nxt, nitems, items, rchunk);
    auto ctab = [&](const ChunkPos &q) { return rtab + (int64_t)q.ch * (TROWS * TP); };
    // prologue: indices of the first chunk, then its records and the next chunk's indices
    if (cur.item >= 0) stage_idx(sidx[0], pairs, cur.q0, min(TK, cur.it.z - cur.q0), tid);
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    bld_sync();
    if (cur.item >= 0)
      stage_chunk<CC, VEC>(usm + L::OFF_STAGE, sidx[0], min(TK, cur.it.z - cur.q0), tid, C, c0, nc, ctab(cur), yw);
    if (nxt.item >= 0) stage_idx(sidx[1], pairs, nxt.q0, min(TK, nxt.it.z - nxt.q0), tid);
    asm volatile("cp.async.commit_group;\n" ::);
    int c = 0;  // chunks walked (staging buffers alternate per chunk)
    int m = 0;  // chunks handed to the MMA warp (accumulator slots alternate per handed chunk)
    while (cur.item >= 0) {
      const int nq = min(TK, cur.it.z - cur.q0);
      const bool last = cur.q0 + TK >= cur.it.z;
      const ChunkPos nxt3 = next_chunk(nxt2, nitems, items, rchunk);
      // records of chunk c and indices of chunk c + 1 have landed
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      bld_sync();
      if (nxt.item >= 0)
        stage_chunk<CC, VEC>(usm + L::OFF_STAGE + ((c + 1) & 1) * L::STAGE, sidx[(c + 1) % 3],
                             min(TK, nxt.it.z - nxt.q0), tid, C, c0, nc, ctab(nxt), yw);
      if (nxt2.item >= 0) stage_idx(sidx[(c + 2) % 3], pairs, nxt2.q0, min(TK, nxt2.it.z - nxt2.q0), tid);
      asm volatile("cp.async.commit_group;\n" ::);
      ++c;
      if (nq == 0) {
        // an item without pairs: its region is zero (a split region was zeroed beforehand)
        if (!cur.it.w) write_region(cur.it.x, false, true);
      } else {
        const unsigned char *stg = usm + L::OFF_STAGE + ((c - 1) & 1) * L::STAGE;
        const float *sv = reinterpret_cast<const float *>(stg);
        const float *tb = reinterpret_cast<const float *>(stg + L::SV);
        const int slot = m & 1;
        // ---- the slot is free once its chunk (two back) is summed ----
        if (!retire(slot)) {
          ok = false;
          break;
        }
        const int nks = (nq + 7) >> 3;  // k-steps with pairs
        // ---- W: this thread's row, k-steps wg, wg + 4, wg + 8, hi and lo, into tensor memory ----
        {
          const float *ryz = tb + (pz * 4 + py) * TP, *rxx = tb + (16 + px) * TP;
          const uint32_t ta = lane_base + (uint32_t)(L::A0 + 2 * TK * slot);
#pragma unroll
          for (int h = 0; h < TK / 32; h++) {
            const int ks = wg + 4 * h;
            if (ks < nks) {
              const float4 a0 = *reinterpret_cast<const float4 *>(ryz + 8 * ks);
              const float4 a1 = *reinterpret_cast<const float4 *>(ryz + 8 * ks + 4);
              const float4 b0 = *reinterpret_cast<const float4 *>(rxx + 8 * ks);
              const float4 b1 = *reinterpret_cast<const float4 *>(rxx + 8 * ks + 4);
              const float w[8] = {__fmul_rn(a0.x, b0.x), __fmul_rn(a0.y, b0.y), __fmul_rn(a0.z, b0.z),
                                  __fmul_rn(a0.w, b0.w), __fmul_rn(a1.x, b1.x), __fmul_rn(a1.y, b1.y),
                                  __fmul_rn(a1.z, b1.z), __fmul_rn(a1.w, b1.w)};
              uint32_t hh[8], ll[8];
#pragma unroll
              for (int i = 0; i < 8; i++) {
                hh[i] = hi_bits(w[i]);
                ll[i] = __float_as_uint(w[i] - __uint_as_float(hh[i]));
              }
              tst8(ta + 8 * ks, hh);
              tst8(ta + TK + 8 * ks, ll);
            }
          }
        }
        // ---- V: K-major canonical, hi and lo, into the slot's shared buffers ----
        {
          // (n, 4 consecutive k) units; NBLD is a multiple of N, so a thread keeps its n
          static_assert(NBLD % N == 0, "one column per thread");
          const int n = tid % N;
          unsigned char *bh = usm + L::OFF_B + slot * 2 * L::BOP + canon(n, 0);
          const float *sp = sv + n;
          for (int k4 = tid / N; k4 < 2 * nks; k4 += NBLD / N) {
            const float *q = sp + 4 * k4 * N;
            const float v[4] = {q[0], q[N], q[2 * N], q[3 * N]};
            uint32_t hh[4], ll[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
              hh[i] = hi_bits(v[i]);
              ll[i] = __float_as_uint(v[i] - __uint_as_float(hh[i]));
            }
            *reinterpret_cast<uint4 *>(bh + k4 * 128) = make_uint4(hh[0], hh[1], hh[2], hh[3]);
            *reinterpret_cast<uint4 *>(bh + L::BOP + k4 * 128) = make_uint4(ll[0], ll[1], ll[2], ll[3]);
          }
        }
        if (tid == 0) slot_nks[slot] = nks;
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(s_u32(&full[slot]));
        const unsigned b = 1u << slot;
        outstanding |= b;
        slast = last ? (slast | b) : (slast & ~b);
        ssplit = cur.it.w ? (ssplit | b) : (ssplit & ~b);
        if (slot) org1 = cur.it.x; else org0 = cur.it.x;
        ++m;
      }
      cur = nxt;
      nxt = nxt2;
      nxt2 = nxt3;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    // sum and write what is still in flight (the older chunk first)
    if (ok && (!retire(m & 1) || !retire((m & 1) ^ 1))) ok = false;
    if (ok) {
      // both slots are retired: tell the MMA warp to stop
      if (tid == 0) slot_nks[m & 1] = -1;
      __syncwarp();
      if ((tid & 31) == 0) mbar_arrive(s_u32(&full[m & 1]));
    } else {
      flag_wait_error(g);
      // let MMAs still in flight finish before the tensor memory is freed: the MMA warp
      // either issued a slot's MMAs and their commit, which arrive within microseconds, or
      // gave up before it, so this wait has at least the default limit whatever the plan's
      const long long lim = g.wait_ns > MRG_DEFAULT_WAIT_NS ? g.wait_ns : MRG_DEFAULT_WAIT_NS;
      for (int s = 0; s < 2; s++)
        if ((outstanding >> s) & 1u) mbar_wait(s_u32(&done[s]), (dphase >> s) & 1u, lim);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::TCOLS));
}

}  // namespace

bool umma_supported(int C) { return C >= 8; }
// region origins packed in 11 + 11 + 10 bits
bool umma_grid_fits(const int S[3]) { return S[0] <= 2048 && S[1] <= 2048 && S[2] <= 1024; }
int umma_default_cc(int C) { return C > 16 ? 32 : (C > 8 ? 16 : 8); }

int64_t umma_table_floats() { return (int64_t)TROWS * TP; }

mrg_status launch_item_chunks(const FrameTraj &ft, int *cnt, cudaStream_t st) {
  if (ft.regions.nitems == 0) return MRG_OK;
  k_item_chunks<<<grid_blocks(ft.regions.nitems, 256), 256, 0, st>>>(ft.regions.nitems, ft.regions.items, cnt);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status launch_region_tables(const FrameTraj &ft, cudaStream_t st) {
  const int n = ft.regions.nitems;
  if (n == 0) return MRG_OK;
  k_region_tables<<<std::min(n, 64 * device_sms()), 128, 0, st>>>(n, ft.regions.items, ft.regions.pairs, ft.rchunk,
                                                                   ft.swt, ft.sst, ft.rtab);
  MRG_LAUNCHED();
  return MRG_OK;
}

int read_wait_error(const GridConst &gc) {
  if (!gc.err) return 0;
  int h = 0;
  if (cudaMemcpy(&h, gc.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return h;
}

template <int CC>
static mrg_status launch_umma_cc(const GridConst &gc, const FrameTraj &ft, const float2 *yw, float2 *grid,
                                 cudaStream_t st) {
  typedef TcLayout<CC> L;
  const bool vec = (gc.C % 2 == 0) && (((uintptr_t)yw & 15) == 0) && (((uintptr_t)grid & 15) == 0);
  static DeviceOnce once;
  MRG_TRY(device_once(once, []() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_grid_umma<CC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::TOTAL));
    MRG_CUDA(cudaFuncSetAttribute(k_grid_umma<CC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::TOTAL));
    return MRG_OK;
  }));
  const int sms = device_sms();
  // one CTA per SM (its shared memory keeps a second one off the SM, so the 512 TMEM
  // columns it allocates are always free); every coil pass gets its share of the SMs
  const int npass = (gc.C + CC - 1) / CC;
  const int nx = std::max(1, std::min(ft.regions.nitems, std::max(1, sms / npass)));
  const dim3 blocks((unsigned)nx, (unsigned)npass);
  if (vec)
    k_grid_umma<CC, true><<<blocks, NTHR, L::TOTAL, st>>>(gc, ft.regions.nitems, ft.regions.items, ft.regions.pairs,
                                                          ft.rchunk, ft.rtab, yw, grid);
  else
    k_grid_umma<CC, false><<<blocks, NTHR, L::TOTAL, st>>>(gc, ft.regions.nitems, ft.regions.items,
                                                           ft.regions.pairs, ft.rchunk, ft.rtab, yw, grid);
  MRG_LAUNCHED();
  return MRG_OK;
}

mrg_status pack_region_items(const GridConst &gc, PairSet &ps, cudaStream_t st) {
  if (ps.nitems == 0) return MRG_OK;
  k_pack_regions<<<grid_blocks(ps.nitems, 256), 256, 0, st>>>(region_shape(gc), ps.nitems, ps.items);
  MRG_LAUNCHED();
  return MRG_OK;
}

// The caller zeroes the split regions (ft.regions.split) first.
mrg_status launch_grid_umma(const GridConst &gc, const FrameTraj &ft, int cc, const float2 *yw, float2 *grid,
                            cudaStream_t st) {
  if (!umma_supported(gc.C) || !ft.regions.built || (ft.regions.nitems > 0 && ft.rtab == nullptr)) {
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
