// Kernels of the batched strided FFT passes, shared by the translation units that
// instantiate them for different line lengths (fft.cu, fft_large.cu, fft_large2.cu).
//
// Replaces the per-axis line FFTs of NDarray::fft3 (src/ArrayTemplates.cpp:276-427)
// as used by gridFFT::do_fft / do_ifft (src/gridFFT.cpp:645-711): every axis is
// transformed with FFTW's sign convention (forward = exp(-i...)) and scaled by
// 1/sqrt(S).  The E side is pruned (only the crop of the image is non-zero) and
// the E^H side only produces the crop it keeps, which is exact because the
// dropped inputs are zero and the dropped outputs are never read.
//
// One CTA transforms IB lines (consecutive "inner" elements, coalesced rows of
// IB complex values) of length S = R*Q held in shared memory as [S][IB+1].
// Each line is split S = R x Q (four-step): R-point DFTs across the R threads
// of a line, a twiddle, then a Q-point DFT in registers per thread (radices 2,
// 3, 4, 5 and direct DFTs of larger primes).  R = 8 up to 384 points; longer lines
// (N > 256 at the default 1.5x) take R = 16, so Q stays within the registers.  Twiddles exp(-2 pi i m / S) are computed on the host in double,
// staged in shared memory per CTA and read as broadcasts.
#pragma once

#include <algorithm>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "mrg_internal.h"

namespace mrg {

// per-size twiddle tables exp(-2 pi i m / S), m < S, built once per device (fft.cu)
// Twiddle table of length-S lines on the current device (fft_init_device builds them).
constexpr int kTwDevices = 64;
const float2 *fft_twiddles(int S);

// lengths 192..288 (fft_large.cu), 320..384 (fft_large2.cu) and 400..768 (fft_long.cu)
mrg_status launch_fft_192_288(const FftPass &p, cudaStream_t st);
mrg_status launch_fft_320_384(const FftPass &p, cudaStream_t st);
mrg_status launch_fft_long(const FftPass &p, cudaStream_t st);

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// SIGN * i * a
template <int SIGN>
__device__ __forceinline__ float2 imul(float2 a) {
  return SIGN > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <int SIGN>
__device__ __forceinline__ float2 twid(const float2 *tw, int m) {
  float2 w = tw[m];
  if (SIGN > 0) w.y = -w.y;
  return w;
}

// t[q] <- sum_p t[p] * exp(SIGN*2*pi*i*p*q/P)
template <int P, int SIGN>
__device__ __forceinline__ void bfly(float2 (&t)[P]) {
  if constexpr (P == 2) {
    float2 a = t[0], b = t[1];
    t[0] = cadd(a, b);
    t[1] = csub(a, b);
  } else if constexpr (P == 3) {
    const float h = 0.86602540378443864676f;
    float2 s = cadd(t[1], t[2]), d = csub(t[1], t[2]);
    float2 m = make_float2(t[0].x - 0.5f * s.x, t[0].y - 0.5f * s.y);
    float2 r = imul<SIGN>(make_float2(h * d.x, h * d.y));
    t[0] = cadd(t[0], s);
    t[1] = cadd(m, r);
    t[2] = csub(m, r);
  } else if constexpr (P == 4) {
    float2 a = cadd(t[0], t[2]), b = csub(t[0], t[2]);
    float2 c = cadd(t[1], t[3]), d = imul<SIGN>(csub(t[1], t[3]));
    t[0] = cadd(a, c);
    t[2] = csub(a, c);
    t[1] = cadd(b, d);
    t[3] = csub(b, d);
  } else if constexpr (P == 5) {
    const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
    const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
    const float2 a1 = cadd(t[1], t[4]), a2 = cadd(t[2], t[3]);
    const float2 b1 = csub(t[1], t[4]), b2 = csub(t[2], t[3]);
    const float2 m1 = make_float2(t[0].x + c1 * a1.x + c2 * a2.x, t[0].y + c1 * a1.y + c2 * a2.y);
    const float2 m2 = make_float2(t[0].x + c2 * a1.x + c1 * a2.x, t[0].y + c2 * a1.y + c1 * a2.y);
    const float2 r1 = imul<SIGN>(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
    const float2 r2 = imul<SIGN>(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
    t[0] = cadd(t[0], cadd(a1, a2));
    t[1] = cadd(m1, r1);
    t[4] = csub(m1, r1);
    t[2] = cadd(m2, r2);
    t[3] = csub(m2, r2);
  } else {
    static_assert(P == 2 || P == 3 || P == 4 || P == 5, "radix");
  }
}

// DFT of odd prime length P >= 7 from symmetric pairs: with a_j = t_j + t_{P-j},
// b_j = t_j - t_{P-j}, X_k = t_0 + sum_j cos(2 pi jk/P) a_j + SIGN i sum_j sin(2 pi jk/P) b_j
// and X_{P-k} the same with the sine term negated.  cos and sin come from the length-S
// table (tw[m] = exp(-2 pi i m / S), S a multiple of P).
template <int P, int SIGN, int S>
__device__ __forceinline__ void bfly_prime(float2 (&t)[P], const float2 *tw) {
  constexpr int H = (P - 1) / 2;
  float2 a[H], b[H];
#pragma unroll
  for (int j = 1; j <= H; j++) {
    a[j - 1] = cadd(t[j], t[P - j]);
    b[j - 1] = csub(t[j], t[P - j]);
  }
  const float2 t0 = t[0];
  float2 s = t0;
#pragma unroll
  for (int j = 0; j < H; j++) s = cadd(s, a[j]);
  t[0] = s;
#pragma unroll
  for (int k = 1; k <= H; k++) {
    float2 m = t0, r = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 1; j <= H; j++) {
      const float2 w = tw[((j * k) % P) * (S / P)];  // (cos, -sin)
      m = make_float2(m.x + w.x * a[j - 1].x, m.y + w.x * a[j - 1].y);
      r = make_float2(r.x - w.y * b[j - 1].x, r.y - w.y * b[j - 1].y);
    }
    const float2 ir = imul<SIGN>(r);
    t[k] = cadd(m, ir);
    t[P - k] = csub(m, ir);
  }
}

// radix of the first decimation step: 4, 2, 3, 5, then the smallest prime factor
constexpr int first_factor(int q) {
  if (q % 4 == 0) return 4;
  if (q % 2 == 0) return 2;
  if (q % 3 == 0) return 3;
  if (q % 5 == 0) return 5;
  for (int f = 7; f < q; f += 2)
    if (q % f == 0) return f;
  return q;
}

// In-register DFT of length Q (decimation in time), natural order in and out;
// tw is the length-S table, S a multiple of Q.
template <int Q, int SIGN, int S>
__device__ __forceinline__ void reg_fft(float2 (&v)[Q], const float2 *tw) {
  if constexpr (Q == 1) {
    return;
  } else {
    constexpr int P = first_factor(Q);
    constexpr int Q2 = Q / P;
    float2 sub[P][Q2];
#pragma unroll
    for (int p = 0; p < P; p++)
#pragma unroll
      for (int m = 0; m < Q2; m++) sub[p][m] = v[p + P * m];
#pragma unroll
    for (int p = 0; p < P; p++) reg_fft<Q2, SIGN, S>(sub[p], tw);
#pragma unroll
    for (int k = 0; k < Q2; k++) {
      float2 t[P];
#pragma unroll
      for (int p = 0; p < P; p++) t[p] = (p * k == 0) ? sub[p][k] : cmul(sub[p][k], twid<SIGN>(tw, p * k * (S / Q)));
      if constexpr (P <= 5)
        bfly<P, SIGN>(t);
      else
        bfly_prime<P, SIGN, S>(t, tw);
#pragma unroll
      for (int q = 0; q < P; q++) v[k + Q2 * q] = t[q];
    }
  }
}

// Deapodisation weight of element l of line (o, i), the reference's (winz * winy) * winx
// (src/gridFFT.cpp:972-986, :926-941): per-line factor `lw` from line_weight, then
// elem_weight for the element.
__device__ __forceinline__ float line_weight(const FftPass &p, int64_t o, int64_t i) {
  if (p.wmode) return p.wo[o / p.wdiv] * p.wi[o % p.wdiv];  // winz * winy of the line's row
  return 0.0f;
}
__device__ __forceinline__ float elem_weight(const FftPass &p, float lw, float wl_l, int64_t o, int64_t i) {
  if (p.wmode) return lw * wl_l;                  // (winz * winy) * winx
  return (wl_l * p.wo[o]) * p.wi[i / p.C];         // (winz * winy) * winx along z
}

// P: shared-memory row pitch when it is a compile-time constant (IB = P lines, no
// padding), else 0 (pitch and IB from the pass).  With P fixed every shared-memory
// address in the transform steps is the thread's base plus a constant.
template <int Q, int SIGN, int MODE, int P, int R = 8>
__global__ void __launch_bounds__(256, 2) k_fft(const FftPass p) {
  constexpr int S = R * Q;
  extern __shared__ float2 sm[];  // [S][IBp] data, then S twiddles
  const int IB = P ? P : p.IB;
  const int IBp = P ? P : (p.lfast ? p.IB + 1 : p.IB);  // pad only for column-wise (contiguous-line) access
  const int tid = threadIdx.x;
  float2 *tw = sm + S * (IB + 1);
  for (int m = tid; m < S; m += blockDim.x) tw[m] = p.tw[m];
  const int j = tid % IB, t = tid / IB;  // R threads per line
  // Line (o, i) of the CTA's IB lines.  When inner % IB == 0 (nib = inner / IB) every line
  // of the CTA shares o and one 32-bit division per thread finds it.
  int64_t o0 = 0, i0 = 0;
  if (p.nib) {
    const unsigned b = blockIdx.x, ob = b / (unsigned)p.nib;
    o0 = ob;
    i0 = (int64_t)(b - ob * (unsigned)p.nib) * IB;
  }
  const int64_t line = (int64_t)blockIdx.x * IB + j;
  const bool lv = line < p.nlines;
  int64_t o = 0, i = 0;
  if (p.nib) {
    o = o0;
    i = i0 + j;
  } else if (lv) {
    o = line / p.inner;
    i = line - o * p.inner;
  }
  float2 *col = sm + j;  // this thread's column

  // ---- load (zero rows outside [in_off, in_off + Lin)) ----
  if (p.vec16 && !(MODE == FFT_SETIMG && !p.has_smap)) {
    // 16-byte asynchronous copies (two adjacent lines per copy), many in flight
    const int npair = IB >> 1;
    const int jp = tid % npair, r0 = tid / npair, rstep = blockDim.x / npair;
    const int64_t ln = (int64_t)blockIdx.x * IB + 2 * jp;
    const bool pv = ln < p.nlines;
    int64_t po = 0, pi = 0;
    if (p.nib) {
      po = o0;
      pi = i0 + 2 * jp;
    } else if (pv) {
      po = ln / p.inner;
      pi = ln - po * p.inner;
    }
    const float2 *src = (MODE == FFT_SETIMG) ? p.smap : p.in;
    const float2 *gs = src + po * p.in_os + pi + (int64_t)r0 * p.in_ls;
    const int64_t gstep = (int64_t)rstep * p.in_ls;
    unsigned sa = (unsigned)__cvta_generic_to_shared(sm + (r0 + p.in_off) * IBp + 2 * jp);
    const unsigned sstep = (unsigned)(rstep * IBp * (int)sizeof(float2));
    if (pv) {
      for (int li = r0; li < p.Lin; li += rstep, gs += gstep, sa += sstep)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gs));
    } else {
      for (int li = r0; li < p.Lin; li += rstep)
        *reinterpret_cast<float4 *>(sm + (li + p.in_off) * IBp + 2 * jp) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int e = tid; e < (S - p.Lin) * IB; e += blockDim.x) {
      const int jj = e % IB, k = e / IB;
      const int r = (k < p.in_off) ? k : k + p.Lin;
      sm[r * IBp + jj] = make_float2(0.f, 0.f);
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();
    if constexpr (MODE == FFT_SETIMG) {
      // image = (winz*winy)*winx * X * smap  (src/gridFFT.cpp:972-986); smap already in smem
      if (lv) {
        const int64_t ib = o * p.in_os + i;
        const float lw = line_weight(p, o, i);
        const int64_t xb = ib / p.C, xs = p.in_ls / p.C;  // X has no coil axis
        for (int l0 = t; l0 < p.Lin; l0 += 8 * R) {
          float2 xv[8];
          float wv[8];
#pragma unroll
          for (int k = 0; k < 8; k++) {  // 8 independent loads in flight
            const int li = l0 + R * k;
            if (li < p.Lin) {
              xv[k] = __ldg(p.X + xb + (int64_t)li * xs);
              wv[k] = __ldg(p.wl + li);
            }
          }
#pragma unroll
          for (int k = 0; k < 8; k++) {
            const int li = l0 + R * k;
            if (li < p.Lin) {
              const float w = elem_weight(p, lw, wv[k], o, i);
              float2 *d = col + (li + p.in_off) * IBp;
              *d = cmul(make_float2(w * xv[k].x, w * xv[k].y), *d);
            }
          }
        }
      }
      __syncthreads();
    }
  } else if (!p.lfast) {
    const int64_t ib = o * p.in_os + i;
    for (int r = t; r < S; r += R) {
      float2 v = make_float2(0.f, 0.f);
      const int li = r - p.in_off;
      if (lv && li >= 0 && li < p.Lin) {
        const int64_t off = ib + (int64_t)li * p.in_ls;
        if constexpr (MODE == FFT_SETIMG) {
          const int64_t vox = off / p.C;
          const float w = elem_weight(p, line_weight(p, o, i), p.wl[li], o, i);
          const float2 x = p.X[vox];
          v = make_float2(w * x.x, w * x.y);
          if (p.has_smap) v = cmul(v, p.smap[off]);
        } else {
          v = p.in[off];
        }
      }
      col[r * IBp] = v;
    }
    __syncthreads();
  } else {
    // inner == 1 and in_ls == 1: each line is contiguous; sweep along lines.
    const int64_t l0 = (int64_t)blockIdx.x * IB;
    for (int e = tid; e < S * IB; e += blockDim.x) {
      const int jj = e / S, r = e - jj * S;
      float2 v = make_float2(0.f, 0.f);
      const int li = r - p.in_off;
      const int64_t ln = l0 + jj;
      if (ln < p.nlines && li >= 0 && li < p.Lin) v = p.in[ln * p.in_os + li];
      sm[r * IBp + jj] = v;
    }
    __syncthreads();
  }

  // ---- step A: R-point DFTs over n1 (rows Q*n1 + n2), twiddle W_S^(n2*k1) ----
  for (int n2 = t; n2 < Q; n2 += R) {
    float2 a[R];
    float2 *c2 = col + n2 * IBp;
#pragma unroll
    for (int n1 = 0; n1 < R; n1++) a[n1] = c2[Q * n1 * IBp];
    reg_fft<R, SIGN, S>(a, tw);
#pragma unroll
    for (int k1 = 1; k1 < R; k1++) a[k1] = cmul(a[k1], twid<SIGN>(tw, n2 * k1));
#pragma unroll
    for (int k1 = 0; k1 < R; k1++) c2[Q * k1 * IBp] = a[k1];
  }
  __syncthreads();

  // ---- step C: Q-point DFT of rows Q*t .. Q*t+Q-1 -> rows t + R*k2 ----
  {
    float2 v[Q];
    const float2 *cq = col + Q * t * IBp;
#pragma unroll
    for (int n2 = 0; n2 < Q; n2++) v[n2] = cq[n2 * IBp];
    reg_fft<Q, SIGN, S>(v, tw);
    __syncthreads();
    float2 *ct = col + t * IBp;
#pragma unroll
    for (int k2 = 0; k2 < Q; k2++) ct[R * k2 * IBp] = v[k2];
  }
  __syncthreads();

  // ---- store ----
  if constexpr (MODE != FFT_ACCUM) {
    if (p.vec16o) {
      const int npair = IB >> 1;
      const int jp = tid % npair, r0 = tid / npair, rstep = blockDim.x / npair;
      const int64_t ln = (int64_t)blockIdx.x * IB + 2 * jp;
      if (ln < p.nlines) {
        int64_t po, pi;
        if (p.nib) {
          po = o0;
          pi = i0 + 2 * jp;
        } else {
          po = ln / p.inner;
          pi = ln - po * p.inner;
        }
        float4 *ob = reinterpret_cast<float4 *>(p.out + po * p.out_os + pi + (int64_t)r0 * p.out_ls);
        const int64_t ostep = (int64_t)rstep * (p.out_ls / 2);
        const float4 *sv = reinterpret_cast<const float4 *>(sm + (r0 + p.out_off) * IBp + 2 * jp);
        const int svstep = rstep * IBp / 2;
        const float sc = p.scale;
#pragma unroll 4
        for (int r = r0; r < p.Lout; r += rstep, ob += ostep, sv += svstep) {
          const float4 v = *sv;
          *ob = make_float4(v.x * sc, v.y * sc, v.z * sc, v.w * sc);
        }
      }
    } else if (!p.lfast) {
      if (lv) {
        const int64_t ob = o * p.out_os + i;
        for (int r = t; r < p.Lout; r += R) {
          float2 v = col[(r + p.out_off) * IBp];
          p.out[ob + (int64_t)r * p.out_ls] = make_float2(v.x * p.scale, v.y * p.scale);
        }
      }
    } else {
      const int64_t l0 = (int64_t)blockIdx.x * IB;
      for (int e = tid; e < p.Lout * IB; e += blockDim.x) {
        const int jj = e / p.Lout, r = e - jj * p.Lout;
        const int64_t ln = l0 + jj;
        if (ln < p.nlines) {
          float2 v = sm[(r + p.out_off) * IBp + jj];
          p.out[ln * p.out_os + r] = make_float2(v.x * p.scale, v.y * p.scale);
        }
      }
    }
  } else {
    // X += sum_c (wl*wo*wi) * v * conj(smap)   (gridFFT::accumulate, src/gridFFT.cpp:926-941)
    const int C = p.C;
    if (lv) {
      const int64_t sb = o * p.out_os + i;
      const float lw = line_weight(p, o, i);
      for (int r0 = t; r0 < p.Lout; r0 += 8 * R) {
        float2 sv[8];
        float wv[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {  // 8 independent smap loads in flight
          const int r = r0 + R * k;
          if (r < p.Lout) {
            sv[k] = p.has_smap ? __ldg(p.smap + sb + (int64_t)r * p.out_ls) : make_float2(1.f, 0.f);
            wv[k] = __ldg(p.wl + r);
          }
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int r = r0 + R * k;
          if (r >= p.Lout) continue;
          float2 v = col[(r + p.out_off) * IBp];
          v = make_float2(v.x * p.scale, v.y * p.scale);
          const float w = elem_weight(p, lw, wv[k], o, i);
          v = make_float2(w * v.x, w * v.y);
          if (p.has_smap) {
            float2 s2 = sv[k];
            s2.y = -s2.y;
            v = cmul(v, s2);
          }
          if (p.acc_atomic) {
            float2 *dst = p.acc + (int64_t)r * p.acc_l + o * p.acc_o + i / C;
            atomicAdd(&dst->x, v.x);
            atomicAdd(&dst->y, v.y);
          } else {
            col[(r + p.out_off) * IBp] = v;
          }
        }
      }
    }
    if (!p.acc_atomic) {
      __syncthreads();
      // IB is a multiple of C: the C lines of one voxel are consecutive in this CTA.
      const int G = IB / C;
      const int64_t line0 = (int64_t)blockIdx.x * IB;
      for (int e = tid; e < p.Lout * G; e += blockDim.x) {
        const int g = e % G, r = e / G;
        const int64_t ln = line0 + (int64_t)g * C;
        if (ln >= p.nlines) continue;
        int64_t oo, ii;
        if (p.nib) {
          oo = o0;
          ii = i0 + (int64_t)g * C;
        } else {
          oo = ln / p.inner;
          ii = ln - oo * p.inner;
        }
        // rotated start (coil (c + r) mod C at step c): the rows of neighbouring threads sit
        // IBp apart, a multiple of the 32 banks, so the same coil index would hit one bank
        float2 s = make_float2(0.f, 0.f);
        const float2 *row = sm + (r + p.out_off) * IBp + g * C;
        int cc = r % C;
        for (int c = 0; c < C; c++) {
          s = cadd(s, row[cc]);
          cc = (cc + 1 == C) ? 0 : cc + 1;
        }
        float2 *dst = p.acc + (int64_t)r * p.acc_l + oo * p.acc_o + ii / C;
        float2 cur = *dst;
        *dst = cadd(cur, s);
      }
    }
  }
}

// Plain passes, persistent: a CTA walks tiles of IB lines (IB = P, no tile straddles an
// outer row, 16-byte line-pair copies).  Once the Q-point step has read a tile's rows into
// registers, the next tile's copies are issued into the same shared memory, so they run
// while this tile is transformed and stored (straight from registers, rows t + 8 k2 of
// line j: IB lines x 8 bytes contiguous per row).
template <int Q, int SIGN, int P, int R = 8>
__global__ void __launch_bounds__(R * P) k_fft_pp(const FftPass p, int ntiles) {
  constexpr int S = R * Q, IB = P, NPAIR = IB / 2;
  extern __shared__ float2 sm[];  // [S][IB] data, then S twiddles
  float2 *tw = sm + S * (IB + 1);
  const int tid = threadIdx.x;
  for (int m = tid; m < S; m += blockDim.x) tw[m] = p.tw[m];
  const int j = tid % IB, t = tid / IB;
  float2 *col = sm + j;
  const int jp = tid % NPAIR, r0 = tid / NPAIR, rstep = blockDim.x / NPAIR;
  const unsigned nib = (unsigned)p.nib;
  auto issue = [&](int tile) {
    const unsigned ob = (unsigned)tile / nib;
    const int64_t i0 = (int64_t)((unsigned)tile - ob * nib) * IB;
    const float2 *gs = p.in + (int64_t)ob * p.in_os + i0 + 2 * jp + (int64_t)r0 * p.in_ls;
    const int64_t gstep = (int64_t)rstep * p.in_ls;
    unsigned sa = (unsigned)__cvta_generic_to_shared(sm + (r0 + p.in_off) * IB + 2 * jp);
    const unsigned sstep = (unsigned)(rstep * IB * (int)sizeof(float2));
    for (int li = r0; li < p.Lin; li += rstep, gs += gstep, sa += sstep)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gs));
    for (int e = tid; e < (S - p.Lin) * IB; e += blockDim.x) {
      const int jj = e % IB, k = e / IB;
      const int r = (k < p.in_off) ? k : k + p.Lin;
      sm[r * IB + jj] = make_float2(0.f, 0.f);
    }
    asm volatile("cp.async.commit_group;\n" ::);
  };
  int tile = blockIdx.x;
  if (tile < ntiles) issue(tile);
  for (; tile < ntiles; tile += gridDim.x) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    // ---- step A: R-point DFTs over n1 (rows Q*n1 + n2), twiddle W_S^(n2*k1) ----
    for (int n2 = t; n2 < Q; n2 += R) {
      float2 a[R];
      float2 *c2 = col + n2 * IB;
#pragma unroll
      for (int n1 = 0; n1 < R; n1++) a[n1] = c2[Q * n1 * IB];
      reg_fft<R, SIGN, S>(a, tw);
#pragma unroll
      for (int k1 = 1; k1 < R; k1++) a[k1] = cmul(a[k1], twid<SIGN>(tw, n2 * k1));
#pragma unroll
      for (int k1 = 0; k1 < R; k1++) c2[Q * k1 * IB] = a[k1];
    }
    __syncthreads();
    // ---- step C: rows Q*t .. Q*t+Q-1 into registers; then the buffer is free ----
    float2 v[Q];
    const float2 *cq = col + Q * t * IB;
#pragma unroll
    for (int n2 = 0; n2 < Q; n2++) v[n2] = cq[n2 * IB];
    __syncthreads();
    if (tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x);
    reg_fft<Q, SIGN, S>(v, tw);
    const unsigned ob = (unsigned)tile / nib;
    const int64_t i = (int64_t)((unsigned)tile - ob * nib) * IB + j;
    float2 *go = p.out + (int64_t)ob * p.out_os + i;
    const float sc = p.scale;
#pragma unroll
    for (int k2 = 0; k2 < Q; k2++) {
      const int r = t + R * k2 - p.out_off;
      if (r >= 0 && r < p.Lout) go[(int64_t)r * p.out_ls] = make_float2(v[k2].x * sc, v[k2].y * sc);
    }
  }
}

// The persistent plain pass with each tile's rows brought in by the tensor-memory
// accelerator: nbox cp.async.bulk.tensor copies of brows rows each (a 3D tensor map over
// (2 inner floats, Lin rows, outer rows), box (2 IB floats, brows, 1): the tile's IB
// lines), their completion counted on one mbarrier instead of every thread issuing 16-byte
// copies.  The mbarrier wait is bounded; a CTA whose wait runs out records it in the
// plan's error word, waits once more for the copies in flight and returns.
__device__ __forceinline__ bool fft_mbar_wait(uint32_t bar, uint32_t parity, long long limit_ns) {
  long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 >= limit_ns) return false;
    __nanosleep(64);
  }
}

template <int Q, int SIGN, int P, int R>
__global__ void __launch_bounds__(R * P) k_fft_pt(const __grid_constant__ CUtensorMap tmap, const FftPass p, int ntiles,
                                                  int nbox, int brows) {
  constexpr int S = R * Q, IB = P;
  extern __shared__ __align__(128) float2 sm[];  // [S][IB] data, S twiddles, the mbarrier
  float2 *tw = sm + S * (IB + 1);
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(tw + S);
  const int tid = threadIdx.x;
  for (int m = tid; m < S; m += blockDim.x) tw[m] = p.tw[m];
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int j = tid % IB, t = tid / IB;
  float2 *col = sm + j;
  const unsigned nib = (unsigned)p.nib;
  const uint32_t bytes = (uint32_t)(nbox * brows * IB * (int)sizeof(float2));
  auto issue = [&](int tile) {
    if (tid == 0) {
      const unsigned ob = (unsigned)tile / nib;
      const int x = 2 * (int)((unsigned)tile - ob * nib) * IB;  // floats: a multiple of 32
      // the buffer's earlier generic reads (ordered by the barrier before this call) come
      // before the asynchronous writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
      for (int b = 0; b < nbox; b++) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(sm + (p.in_off + b * brows) * IB);
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
            "%4}], [%5];" ::"r"(dst),
            "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(x), "r"(b * brows), "r"((int)ob), "r"(bar)
            : "memory");
      }
    }
    for (int e = tid; e < (S - p.Lin) * IB; e += blockDim.x) {  // rows outside the copied ones
      const int jj = e % IB, k = e / IB;
      const int r = (k < p.in_off) ? k : k + p.Lin;
      sm[r * IB + jj] = make_float2(0.f, 0.f);
    }
  };
  uint32_t phase = 0;
  int tile = blockIdx.x;
  if (tile < ntiles) issue(tile);
  for (; tile < ntiles; tile += gridDim.x) {
    const bool ok = fft_mbar_wait(bar, phase, MRG_DEFAULT_WAIT_NS);
    if (__syncthreads_or(!ok)) {
      if (tid == 0 && p.err) atomicExch(p.err, MRG_WAIT_EXPIRED);
      fft_mbar_wait(bar, phase, MRG_DEFAULT_WAIT_NS);  // the copies in flight land before the CTA leaves
      return;
    }
    phase ^= 1u;
    // ---- step A: R-point DFTs over n1 (rows Q*n1 + n2), twiddle W_S^(n2*k1) ----
    for (int n2 = t; n2 < Q; n2 += R) {
      float2 a[R];
      float2 *c2 = col + n2 * IB;
#pragma unroll
      for (int n1 = 0; n1 < R; n1++) a[n1] = c2[Q * n1 * IB];
      reg_fft<R, SIGN, S>(a, tw);
#pragma unroll
      for (int k1 = 1; k1 < R; k1++) a[k1] = cmul(a[k1], twid<SIGN>(tw, n2 * k1));
#pragma unroll
      for (int k1 = 0; k1 < R; k1++) c2[Q * k1 * IB] = a[k1];
    }
    __syncthreads();
    // ---- step C: rows Q*t .. Q*t+Q-1 into registers; then the buffer is free ----
    float2 v[Q];
    const float2 *cq = col + Q * t * IB;
#pragma unroll
    for (int n2 = 0; n2 < Q; n2++) v[n2] = cq[n2 * IB];
    __syncthreads();
    if (tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x);
    reg_fft<Q, SIGN, S>(v, tw);
    const unsigned ob = (unsigned)tile / nib;
    const int64_t i = (int64_t)((unsigned)tile - ob * nib) * IB + j;
    float2 *go = p.out + (int64_t)ob * p.out_os + i;
    const float sc = p.scale;
#pragma unroll
    for (int k2 = 0; k2 < Q; k2++) {
      const int r = t + R * k2 - p.out_off;
      if (r >= 0 && r < p.Lout) go[(int64_t)r * p.out_ls] = make_float2(v[k2].x * sc, v[k2].y * sc);
    }
  }
}

// Set-image x passes, persistent: the first pass of a multi-coil E, lines along x with the
// coils innermost (inner == C == in_ls), so the IB lines of a tile are IB coils of one
// image row o.  Tiles are walked as in k_fft_pp; beside a tile's maps the copies bring the
// image row X[o][0..Lin), which becomes (w X)[l] in place once it has landed, w = (winz *
// winy) * winx.  The 8-point step multiplies each map value by it as it reads the row
// (src/gridFFT.cpp:972-986: image = (w X) smap).
template <int Q, int P, int R = 8>
__global__ void __launch_bounds__(R * P) k_fft_ps(const FftPass p, int ntiles) {
  constexpr int S = R * Q, IB = P, NPAIR = IB / 2;
  extern __shared__ float2 sm[];  // [S][IB] data, S twiddles, S image row
  float2 *tw = sm + S * (IB + 1);
  float2 *xr = tw + S;
  const int tid = threadIdx.x;
  for (int m = tid; m < S; m += blockDim.x) tw[m] = p.tw[m];
  const int j = tid % IB, t = tid / IB;
  float2 *col = sm + j;
  const int jp = tid % NPAIR, r0 = tid / NPAIR, rstep = blockDim.x / NPAIR;
  const unsigned nib = (unsigned)p.nib;
  const int64_t xos = p.in_os / p.C;  // image row pitch (X has no coil axis)
  auto issue = [&](int tile) {
    const unsigned ob = (unsigned)tile / nib;
    const int64_t i0 = (int64_t)((unsigned)tile - ob * nib) * IB;
    const float2 *gs = p.smap + (int64_t)ob * p.in_os + i0 + 2 * jp + (int64_t)r0 * p.in_ls;
    const int64_t gstep = (int64_t)rstep * p.in_ls;
    unsigned sa = (unsigned)__cvta_generic_to_shared(sm + (r0 + p.in_off) * IB + 2 * jp);
    const unsigned sstep = (unsigned)(rstep * IB * (int)sizeof(float2));
    for (int li = r0; li < p.Lin; li += rstep, gs += gstep, sa += sstep)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gs));
    const float2 *gx = p.X + (int64_t)ob * xos;
    for (int li = tid; li < p.Lin; li += blockDim.x)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(xr + li)),
                   "l"(gx + li));
    for (int e = tid; e < (S - p.Lin) * IB; e += blockDim.x) {
      const int jj = e % IB, k = e / IB;
      const int r = (k < p.in_off) ? k : k + p.Lin;
      sm[r * IB + jj] = make_float2(0.f, 0.f);
    }
    asm volatile("cp.async.commit_group;\n" ::);
  };
  int tile = blockIdx.x;
  if (tile < ntiles) issue(tile);
  for (; tile < ntiles; tile += gridDim.x) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    const unsigned ob = (unsigned)tile / nib;
    {
      const float lw = p.wo[(int64_t)ob / p.wdiv] * p.wi[(int64_t)ob % p.wdiv];  // winz * winy of the row
      for (int li = tid; li < p.Lin; li += blockDim.x) {
        const float w = lw * __ldg(p.wl + li);
        const float2 x = xr[li];
        xr[li] = make_float2(w * x.x, w * x.y);
      }
    }
    __syncthreads();
    // ---- step A with set_image: R-point DFTs over n1 (rows Q*n1 + n2) ----
    for (int n2 = t; n2 < Q; n2 += R) {
      float2 a[R];
      float2 *c2 = col + n2 * IB;
#pragma unroll
      for (int n1 = 0; n1 < R; n1++) {
        a[n1] = c2[Q * n1 * IB];
        const int li = Q * n1 + n2 - p.in_off;
        if ((unsigned)li < (unsigned)p.Lin) a[n1] = cmul(xr[li], a[n1]);
      }
      reg_fft<R, -1, S>(a, tw);
#pragma unroll
      for (int k1 = 1; k1 < R; k1++) a[k1] = cmul(a[k1], twid<-1>(tw, n2 * k1));
#pragma unroll
      for (int k1 = 0; k1 < R; k1++) c2[Q * k1 * IB] = a[k1];
    }
    __syncthreads();
    // ---- step C: rows into registers, then the next tile's copies ----
    float2 v[Q];
    const float2 *cq = col + Q * t * IB;
#pragma unroll
    for (int n2 = 0; n2 < Q; n2++) v[n2] = cq[n2 * IB];
    __syncthreads();
    if (tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x);
    reg_fft<Q, -1, S>(v, tw);
    const int64_t i = (int64_t)((unsigned)tile - ob * nib) * IB + j;
    float2 *go = p.out + (int64_t)ob * p.out_os + i;
    const float sc = p.scale;
#pragma unroll
    for (int k2 = 0; k2 < Q; k2++) {
      const int r = t + R * k2 - p.out_off;
      if (r >= 0 && r < p.Lout) go[(int64_t)r * p.out_ls] = make_float2(v[k2].x * sc, v[k2].y * sc);
    }
  }
}

// Accumulate x passes, persistent: the last pass of a multi-coil E^H, lines along x with
// one tile = the C coils of one outer row o (IB == C == inner == in_ls).  The input tile is
// copied one tile ahead as in k_fft_pp; the maps of the row's Lout output points and the
// row of X are copied (a second group) while the tile is transformed.  Each thread puts
// w v conj(smap) of its coil in place of the map value, then thread r sums row r over the
// coils into X[o][r] (src/gridFFT.cpp:926-941), so the sum needs no atomics.
template <int Q, int P, int R = 8>
__global__ void __launch_bounds__(R * P) k_fft_pa(const FftPass p, int ntiles) {
  constexpr int S = R * Q, IB = P, NPAIR = IB / 2;
  extern __shared__ float2 sm[];  // [S][IB] data, S twiddles, [Lout][IB] maps, Lout values of X
  float2 *tw = sm + S * (IB + 1);
  float2 *mp = tw + S;
  float2 *xa = mp + p.Lout * IB;
  const int tid = threadIdx.x;
  for (int m = tid; m < S; m += blockDim.x) tw[m] = p.tw[m];
  const int j = tid % IB, t = tid / IB;
  float2 *col = sm + j;
  const int jp = tid % NPAIR, r0 = tid / NPAIR, rstep = blockDim.x / NPAIR;
  auto issue_in = [&](int tile) {
    const float2 *gs = p.in + (int64_t)tile * p.in_os + 2 * jp + (int64_t)r0 * p.in_ls;
    const int64_t gstep = (int64_t)rstep * p.in_ls;
    unsigned sa = (unsigned)__cvta_generic_to_shared(sm + (r0 + p.in_off) * IB + 2 * jp);
    const unsigned sstep = (unsigned)(rstep * IB * (int)sizeof(float2));
    for (int li = r0; li < p.Lin; li += rstep, gs += gstep, sa += sstep)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gs));
    for (int e = tid; e < (S - p.Lin) * IB; e += blockDim.x) {
      const int jj = e % IB, k = e / IB;
      const int r = (k < p.in_off) ? k : k + p.Lin;
      sm[r * IB + jj] = make_float2(0.f, 0.f);
    }
  };
  auto issue_maps = [&](int tile) {
    const float2 *gm = p.smap + (int64_t)tile * p.out_os + 2 * jp + (int64_t)r0 * p.out_ls;
    const int64_t gstep = (int64_t)rstep * p.out_ls;
    unsigned sa = (unsigned)__cvta_generic_to_shared(mp + r0 * IB + 2 * jp);
    const unsigned sstep = (unsigned)(rstep * IB * (int)sizeof(float2));
    for (int r = r0; r < p.Lout; r += rstep, gm += gstep, sa += sstep)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gm));
    const float2 *gx = p.acc + (int64_t)tile * p.acc_o;
    for (int r = tid; r < p.Lout; r += blockDim.x)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(xa + r)),
                   "l"(gx + (int64_t)r * p.acc_l));
  };
  // Two commit groups per tile, always committed (empty past the last tile), so that
  // "wait_group 1" always leaves exactly the newest group in flight.
  int tile = blockIdx.x;
  if (tile < ntiles) issue_in(tile);
  asm volatile("cp.async.commit_group;\n" ::);
  if (tile < ntiles) issue_maps(tile);
  asm volatile("cp.async.commit_group;\n" ::);
  for (; tile < ntiles; tile += gridDim.x) {
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this tile's input
    __syncthreads();
    for (int n2 = t; n2 < Q; n2 += R) {
      float2 a[R];
      float2 *c2 = col + n2 * IB;
#pragma unroll
      for (int n1 = 0; n1 < R; n1++) a[n1] = c2[Q * n1 * IB];
      reg_fft<R, +1, S>(a, tw);
#pragma unroll
      for (int k1 = 1; k1 < R; k1++) a[k1] = cmul(a[k1], twid<+1>(tw, n2 * k1));
#pragma unroll
      for (int k1 = 0; k1 < R; k1++) c2[Q * k1 * IB] = a[k1];
    }
    __syncthreads();
    float2 v[Q];
    const float2 *cq = col + Q * t * IB;
#pragma unroll
    for (int n2 = 0; n2 < Q; n2++) v[n2] = cq[n2 * IB];
    __syncthreads();
    const int nxt = tile + (int)gridDim.x;
    if (nxt < ntiles) issue_in(nxt);
    asm volatile("cp.async.commit_group;\n" ::);
    reg_fft<Q, +1, S>(v, tw);
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this tile's maps and X row
    __syncthreads();
    // X += sum_c (winz * winy * winx) v conj(smap)   (gridFFT::accumulate)
    const float lw = p.wo[(int64_t)tile / p.wdiv] * p.wi[(int64_t)tile % p.wdiv];
    const float sc = p.scale;
#pragma unroll
    for (int k2 = 0; k2 < Q; k2++) {
      const int r = t + R * k2 - p.out_off;
      if (r >= 0 && r < p.Lout) {
        float2 val = make_float2(v[k2].x * sc, v[k2].y * sc);
        const float w = lw * __ldg(p.wl + r);
        val = make_float2(w * val.x, w * val.y);
        float2 s2 = mp[r * IB + j];
        s2.y = -s2.y;
        mp[r * IB + j] = cmul(val, s2);
      }
    }
    __syncthreads();
    // rotated start (coil (c + r) mod C at step c) spreads a warp's reads over the banks
    for (int r = tid; r < p.Lout; r += blockDim.x) {
      float2 s = make_float2(0.f, 0.f);
      const float2 *row = mp + r * IB;
      int cc = r % IB;
      for (int c = 0; c < IB; c++) {
        s = cadd(s, row[cc]);
        cc = (cc + 1 == IB) ? 0 : cc + 1;
      }
      p.acc[(int64_t)tile * p.acc_o + (int64_t)r * p.acc_l] = cadd(xa[r], s);
    }
    __syncthreads();
    if (nxt < ntiles) issue_maps(nxt);
    asm volatile("cp.async.commit_group;\n" ::);
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// The accumulate x pass with its copies made by the bulk-copy engine: a tile's input rows
// (S x IB values, contiguous because IB == C == in_ls), the row's maps (Lout x IB) and its
// X row (Lout) are contiguous in memory, so each is one cp.async.bulk copy counted on an
// mbarrier (the input on one, the maps and X row on the other) instead of thousands of
// 16-byte copies.  Otherwise as k_fft_pa.  Waits are bounded; a CTA whose wait runs out
// records it in the plan's error word, waits for what it has in flight and returns.
template <int Q, int P, int R>
__global__ void __launch_bounds__(R * P) k_fft_pb(const FftPass p, int ntiles) {
  constexpr int S = R * Q, IB = P;
  extern __shared__ __align__(128) float2 sm[];  // [S][IB] data, S twiddles, maps, X row, 2 mbarriers
  float2 *tw = sm + S * (IB + 1);
  float2 *mp = tw + S;
  float2 *xa = mp + p.Lout * IB;
  const uint32_t bin = (uint32_t)__cvta_generic_to_shared(xa + p.Lout), bmp = bin + 8;
  const int tid = threadIdx.x;
  for (int m = tid; m < S; m += blockDim.x) tw[m] = p.tw[m];
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bin));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bmp));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int j = tid % IB, t = tid / IB;
  float2 *col = sm + j;
  const uint32_t in_bytes = (uint32_t)(S * IB * (int)sizeof(float2));
  const uint32_t mp_bytes = (uint32_t)(p.Lout * IB * (int)sizeof(float2)), xa_bytes = (uint32_t)(p.Lout * 8);
  auto bulk = [](uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
  };
  auto issue_in = [&](int tile) {
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bin), "r"(in_bytes) : "memory");
      bulk((uint32_t)__cvta_generic_to_shared(sm), p.in + (int64_t)tile * p.in_os, in_bytes, bin);
    }
  };
  auto issue_maps = [&](int tile) {
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bmp), "r"(mp_bytes + xa_bytes)
                   : "memory");
      bulk((uint32_t)__cvta_generic_to_shared(mp), p.smap + (int64_t)tile * p.out_os, mp_bytes, bmp);
      bulk((uint32_t)__cvta_generic_to_shared(xa), p.acc + (int64_t)tile * p.acc_o, xa_bytes, bmp);
    }
  };
  uint32_t ph_in = 0, ph_mp = 0;
  // a wait that ran out: report it, let whatever is in flight land, leave
  auto bail = [&]() {
    if (tid == 0 && p.err) atomicExch(p.err, MRG_WAIT_EXPIRED);
    fft_mbar_wait(bin, ph_in, MRG_DEFAULT_WAIT_NS);
    fft_mbar_wait(bmp, ph_mp, MRG_DEFAULT_WAIT_NS);
  };
  int tile = blockIdx.x;
  if (tile < ntiles) {
    issue_in(tile);
    issue_maps(tile);
  }
  for (; tile < ntiles; tile += gridDim.x) {
    if (__syncthreads_or(!fft_mbar_wait(bin, ph_in, MRG_DEFAULT_WAIT_NS))) {  // this tile's input
      bail();
      return;
    }
    ph_in ^= 1u;
    for (int n2 = t; n2 < Q; n2 += R) {
      float2 a[R];
      float2 *c2 = col + n2 * IB;
#pragma unroll
      for (int n1 = 0; n1 < R; n1++) a[n1] = c2[Q * n1 * IB];
      reg_fft<R, +1, S>(a, tw);
#pragma unroll
      for (int k1 = 1; k1 < R; k1++) a[k1] = cmul(a[k1], twid<+1>(tw, n2 * k1));
#pragma unroll
      for (int k1 = 0; k1 < R; k1++) c2[Q * k1 * IB] = a[k1];
    }
    __syncthreads();
    float2 v[Q];
    const float2 *cq = col + Q * t * IB;
#pragma unroll
    for (int n2 = 0; n2 < Q; n2++) v[n2] = cq[n2 * IB];
    __syncthreads();
    const int nxt = tile + (int)gridDim.x;
    if (nxt < ntiles) issue_in(nxt);
    reg_fft<Q, +1, S>(v, tw);
    if (__syncthreads_or(!fft_mbar_wait(bmp, ph_mp, MRG_DEFAULT_WAIT_NS))) {  // this tile's maps and X row
      bail();
      return;
    }
    ph_mp ^= 1u;
    // X += sum_c (winz * winy * winx) v conj(smap)   (gridFFT::accumulate)
    const float lw = p.wo[(int64_t)tile / p.wdiv] * p.wi[(int64_t)tile % p.wdiv];
    const float sc = p.scale;
#pragma unroll
    for (int k2 = 0; k2 < Q; k2++) {
      const int r = t + R * k2 - p.out_off;
      if (r >= 0 && r < p.Lout) {
        float2 val = make_float2(v[k2].x * sc, v[k2].y * sc);
        const float w = lw * __ldg(p.wl + r);
        val = make_float2(w * val.x, w * val.y);
        float2 s2 = mp[r * IB + j];
        s2.y = -s2.y;
        mp[r * IB + j] = cmul(val, s2);
      }
    }
    __syncthreads();
    for (int r = tid; r < p.Lout; r += blockDim.x) {
      float2 s = make_float2(0.f, 0.f);
      const float2 *row = mp + r * IB;
      int cc = r % IB;
      for (int c = 0; c < IB; c++) {
        s = cadd(s, row[cc]);
        cc = (cc + 1 == IB) ? 0 : cc + 1;
      }
      p.acc[(int64_t)tile * p.acc_o + (int64_t)r * p.acc_l] = cadd(xa[r], s);
    }
    __syncthreads();
    if (nxt < ntiles) issue_maps(nxt);
  }
}

// Persistent launch over ntiles tiles.  The shared-memory cap and the resident CTAs per SM
// (occupancy at the cap, a lower bound for smaller launches of the same kernel) are set up
// once per device; the CTA count is the same on every device of a process.
template <typename K>
static mrg_status launch_persistent(K kern, int threads, size_t smem, size_t smem_cap, DeviceOnce &once, int &ctas,
                                    int ntiles, const FftPass &pp, cudaStream_t st) {
  MRG_TRY(device_once(once, [kern, threads, smem_cap, &ctas]() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cap));
    int c = 0;
    MRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, kern, threads, smem_cap));
    ctas = c < 1 ? 1 : c;
    return MRG_OK;
  }));
  const int nblk = std::max(1, std::min(ntiles, device_sms() * ctas));
  kern<<<nblk, threads, smem, st>>>(pp, ntiles);
  MRG_LAUNCHED();
  return MRG_OK;
}

// R = 8 or 16 threads per line (16: twice the warps per CTA at the same shared memory, for
// the long lines whose tiles leave room for one or two CTAs per SM)
template <int Q, int P, int R = 8>
static mrg_status launch_ps(const FftPass &pp, cudaStream_t st) {
  constexpr int S = R * Q;
  const size_t smem = (size_t)S * (P + 3) * sizeof(float2);
  static DeviceOnce once;
  static int ctas = 1;
  return launch_persistent(k_fft_ps<Q, P, R>, R * P, smem, smem, once, ctas, (int)(pp.nlines / P), pp, st);
}

template <int Q, int P, int R = 8>
static mrg_status launch_pa(const FftPass &pp, cudaStream_t st) {
  constexpr int S = R * Q;
  const size_t smem = ((size_t)S * (P + 2) + (size_t)pp.Lout * (P + 1)) * sizeof(float2);
  const size_t cap = ((size_t)S * (P + 2) + (size_t)S * (P + 1)) * sizeof(float2);
  static DeviceOnce once;
  static int ctas = 1;
  return launch_persistent(k_fft_pa<Q, P, R>, R * P, smem, cap, once, ctas, (int)(pp.nlines / P), pp, st);
}

template <int Q, int P, int R = 8>
static mrg_status launch_pb(const FftPass &pp, cudaStream_t st) {
  constexpr int S = R * Q;
  const size_t smem = ((size_t)S * (P + 2) + (size_t)pp.Lout * (P + 1)) * sizeof(float2) + 16;
  const size_t cap = ((size_t)S * (P + 2) + (size_t)S * (P + 1)) * sizeof(float2) + 16;
  static DeviceOnce once;
  static int ctas = 1;
  return launch_persistent(k_fft_pb<Q, P, R>, R * P, smem, cap, once, ctas, (int)(pp.nlines / P), pp, st);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver
// library); NULL where the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

// The tile copies of a plain persistent pass as tensor-map copies: tiles of IB lines, Lin
// rows in nbox boxes of brows rows (nbox * brows == Lin, brows <= 256).  false where the
// pass's layout does not fit (the caller keeps the 16-byte copies).
inline bool fft_tensor_map(const FftPass &p, int IB, CUtensorMap *map, int *nbox, int *brows) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || p.Lin < 1 || p.inner % IB || (p.nlines % p.inner) || ((uintptr_t)p.in & 15) || (p.in_ls & 1) ||
      (p.in_os & 1))
    return false;
  const int nb = (p.Lin + 255) / 256;
  if (p.Lin % nb) return false;
  const int64_t nouter = p.nlines / p.inner;
  const cuuint64_t dims[3] = {(cuuint64_t)(2 * p.inner), (cuuint64_t)p.Lin, (cuuint64_t)nouter};
  const cuuint64_t strides[2] = {(cuuint64_t)(8 * p.in_ls),
                                 (cuuint64_t)(8 * (nouter > 1 ? p.in_os : p.in_ls * (int64_t)p.Lin))};
  const cuuint32_t box[3] = {(cuuint32_t)(2 * IB), (cuuint32_t)(p.Lin / nb), 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  if (strides[0] % 16 || strides[1] % 16 || strides[0] == 0 || strides[1] == 0) return false;
  if (enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2 *>(p.in), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  *nbox = nb;
  *brows = p.Lin / nb;
  return true;
}

template <int Q, int SIGN, int P, int R>
static mrg_status launch_pt(const FftPass &pp, const CUtensorMap &map, int nbox, int brows, cudaStream_t st) {
  const size_t smem = (size_t)R * Q * (P + 2) * sizeof(float2) + 16;  // + the mbarrier
  static DeviceOnce once;
  static int ctas = 1;
  MRG_TRY(device_once(once, [smem]() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_fft_pt<Q, SIGN, P, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int c = 0;
    MRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_fft_pt<Q, SIGN, P, R>, R * P, smem));
    ctas = c < 1 ? 1 : c;
    return MRG_OK;
  }));
  const int ntiles = (int)(pp.nlines / P);
  const int nblk = std::max(1, std::min(ntiles, device_sms() * ctas));
  k_fft_pt<Q, SIGN, P, R><<<nblk, R * P, smem, st>>>(map, pp, ntiles, nbox, brows);
  MRG_LAUNCHED();
  return MRG_OK;
}

template <int Q, int SIGN, int P, int R = 8>
static mrg_status launch_pp(const FftPass &pp, cudaStream_t st) {
  const size_t smem = (size_t)R * Q * (P + 2) * sizeof(float2);
  static DeviceOnce once;
  static int ctas = 1;  // resident CTAs per SM (the same kernel and shape on every device of a process)
  MRG_TRY(device_once(once, [smem]() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(k_fft_pp<Q, SIGN, P, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int c = 0;
    MRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_fft_pp<Q, SIGN, P, R>, R * P, smem));
    ctas = c < 1 ? 1 : c;
    return MRG_OK;
  }));
  const int sms = device_sms();
  const int ntiles = (int)(pp.nlines / P);
  const int nblk = std::max(1, std::min(ntiles, sms * ctas));
  k_fft_pp<Q, SIGN, P, R><<<nblk, R * P, smem, st>>>(pp, ntiles);
  MRG_LAUNCHED();
  return MRG_OK;
}

// A plain persistent pass with IB = P lines per tile and R threads per line: tensor-map
// copies when the pass asks for them (xp bit 4) and its layout allows, else 16-byte copies.
template <int Q, int P, int R>
static mrg_status launch_plain(const FftPass &pp, cudaStream_t st) {
  if (pp.xp & 4) {
    CUtensorMap map;
    int nbox = 0, brows = 0;
    if (fft_tensor_map(pp, P, &map, &nbox, &brows))
      return pp.sign < 0 ? launch_pt<Q, -1, P, R>(pp, map, nbox, brows, st)
                         : launch_pt<Q, +1, P, R>(pp, map, nbox, brows, st);
  }
  return pp.sign < 0 ? launch_pp<Q, -1, P, R>(pp, st) : launch_pp<Q, +1, P, R>(pp, st);
}

// Q values that get kernels with a compile-time pitch (lines of 192..384 points whose
// factors are 2, 3 and 5; the other lengths run the generic kernel)
constexpr bool fixed_pitch_q(int Q) {
  return Q == 24 || Q == 30 || Q == 32 || Q == 36 || Q == 40 || Q == 45 || Q == 48;
}

template <int Q, int P, int R = 8>
static mrg_status launch_qp(const FftPass &pp, const dim3 grid, const dim3 block, size_t smem, cudaStream_t st) {
  void (*fn)(const FftPass);
  if (pp.mode == FFT_SETIMG) fn = k_fft<Q, -1, FFT_SETIMG, P, R>;
  else if (pp.mode == FFT_ACCUM) fn = k_fft<Q, +1, FFT_ACCUM, P, R>;
  else if (pp.sign < 0) fn = k_fft<Q, -1, FFT_PLAIN, P, R>;
  else fn = k_fft<Q, +1, FFT_PLAIN, P, R>;
  static DeviceOnce once[4];  // per instantiation and mode: set the smem cap once on each device
  const int slot = pp.mode == FFT_PLAIN ? (pp.sign < 0 ? 0 : 1) : (pp.mode == FFT_SETIMG ? 2 : 3);
  MRG_TRY(device_once(once[slot], [fn]() -> mrg_status {
    MRG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  R * Q * (256 / R + 2) * (int)sizeof(float2)));
    return MRG_OK;
  }));
  fn<<<grid, block, smem, st>>>(pp);
  MRG_LAUNCHED();
  return MRG_OK;
}

template <int Q, int R = 8>
static mrg_status launch_q(const FftPass &p, cudaStream_t st) {
  if (p.IB * R > 256) {
    set_error("fft pass: " + std::to_string(p.IB) + " lines per CTA exceed 256 threads for this length");
    return MRG_ERR_INVALID;
  }
  const size_t smem = (size_t)R * Q * (p.IB + 2) * sizeof(float2);
  const int64_t nblk64 = (p.nlines + p.IB - 1) / p.IB;
  if (nblk64 > 0x7fffffff) {
    set_error("fft pass too large");
    return MRG_ERR_UNSUPPORTED;
  }
  const dim3 grid((unsigned)nblk64), block(R * p.IB);
  FftPass pp = p;
  pp.tw = fft_twiddles(R * Q);
  if (!pp.tw) {
    set_error("FFT twiddles not built on this device");
    return MRG_ERR_STATE;
  }
  // CTAs that never straddle an outer row find their row with one 32-bit division
  pp.nib = (p.inner % p.IB == 0 && p.nlines % p.inner == 0) ? (int)(p.inner / p.IB) : 0;
  if constexpr (R == 8 && fixed_pitch_q(Q)) {
    // plain passes whose tiles never straddle an outer row and copy line pairs: persistent
    if (p.mode == FFT_PLAIN && !p.lfast && pp.nib && p.vec16 && p.nlines / p.IB <= 0x7fffffff &&
        (p.IB == 16 || p.IB == 32)) {
      // xp & 3 == 2: 16 threads per line for the lines of 288, 320 and 384 points
      if constexpr (Q == 36 || Q == 40 || Q == 48) {
        if ((p.xp & 3) == 2) return p.IB == 16 ? launch_plain<Q / 2, 16, 16>(pp, st) : launch_plain<Q / 2, 32, 16>(pp, st);
      }
      return p.IB == 16 ? launch_plain<Q, 16, 8>(pp, st) : launch_plain<Q, 32, 8>(pp, st);
    }
    // set_image / accumulate x passes of multi-coil plans (lines along x, coils innermost),
    // persistent when the plan's tuning chose it
    if ((p.xp & 3) && p.wmode == 1 && p.has_smap && pp.nib && p.vec16 && !p.lfast && p.inner == p.C && p.in_ls == p.C &&
        (p.IB == 16 || p.IB == 32) && p.nlines / p.IB <= 0x7fffffff) {
      // xp == 2: 16 threads per line, for the lines of 288, 320 and 384 points
      constexpr bool r16 = (Q == 36 || Q == 40 || Q == 48);
      if (p.mode == FFT_SETIMG && p.in_os % p.C == 0 && p.Lin <= R * Q) {
        if constexpr (r16)
          if ((p.xp & 3) == 2) return p.IB == 16 ? launch_ps<Q / 2, 16, 16>(pp, st) : launch_ps<Q / 2, 32, 16>(pp, st);
        return p.IB == 16 ? launch_ps<Q, 16>(pp, st) : launch_ps<Q, 32>(pp, st);
      }
      if (p.mode == FFT_ACCUM && p.IB == p.C && !p.acc_atomic && p.Lout <= R * Q && p.out_os % 2 == 0 &&
          p.out_ls % 2 == 0 && ((uintptr_t)p.smap & 15) == 0) {
        // xp | 4: the bulk-copy variant, where the tile, the maps and the X row are each contiguous
        const bool bulk = (p.xp & 4) && p.in_off == 0 && p.Lin == R * Q && p.in_ls == p.C && p.out_ls == p.C &&
                          p.acc_l == 1 && p.Lout % 2 == 0 && p.acc_o % 2 == 0 && p.in_os % 2 == 0 &&
                          ((uintptr_t)p.in & 15) == 0 && ((uintptr_t)p.acc & 15) == 0;
        if (bulk) {
          if constexpr (r16)
            if ((p.xp & 3) == 2) return p.IB == 16 ? launch_pb<Q / 2, 16, 16>(pp, st) : launch_pb<Q / 2, 32, 16>(pp, st);
          return p.IB == 16 ? launch_pb<Q, 16>(pp, st) : launch_pb<Q, 32>(pp, st);
        }
        if constexpr (r16)
          if ((p.xp & 3) == 2) return p.IB == 16 ? launch_pa<Q / 2, 16, 16>(pp, st) : launch_pa<Q / 2, 32, 16>(pp, st);
        return p.IB == 16 ? launch_pa<Q, 16>(pp, st) : launch_pa<Q, 32>(pp, st);
      }
    }
    if (!p.lfast && p.IB == 32) return launch_qp<Q, 32>(pp, grid, block, smem, st);
    if (!p.lfast && p.IB == 16) return launch_qp<Q, 16>(pp, grid, block, smem, st);
  }
  return launch_qp<Q, 0, R>(pp, grid, block, smem, st);
}

}  // namespace mrg
