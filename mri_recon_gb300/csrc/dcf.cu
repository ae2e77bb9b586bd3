// Pipe density compensation (RECON::dcf_calc, src/recon_lib.cpp:854-917, with the
// DCFgridFFT gridder, src/DCFgridFFT.cpp): starting from Kw = 1,
//   X   = G Kw          real gridding with the polynomial kernel (forward, :174-277)
//   Kw2 = G^T X         (backward, :323-437)
//   Kw  = |Kw2| < 1e-3 ? 0 : Kw / Kw2                              (:895-905)
// for `iters` rounds, then Kw *= s^3 (scale_kw, :297-321) and Kw = |Kw|.
// The grid has (int)(overgrid * N + 16) points per axis (x's extent from Nz and z's from
// Nx, as recon_lib allocates it), centre S/2, no chop sign;
// a sample's taps are ceil(dk - s*dwin) .. floor(dk + s*dwin) clipped to the grid,
// s = |k|/128*(acc - 1) + 1 widening the kernel with |k|.
//
// One thread per sample: the gridding adds with float atomics (as the reference's
// `omp atomic`), the degridding gathers.  The per-axis weights follow the
// reference's promotions: lut[(int)del]*(1.0 - d) + lut[(int)del+1]*d in double,
// each product rounded to float.
#include "mrg_internal.h"

namespace mrg {

namespace {

struct DcfGeo {
  int S[3];
  float og, dwin, acc;
  const float *lut;
};

struct DcfSample {
  int s[3], e[3];
  float dk[3], sc;
  bool ok;
};

__device__ __forceinline__ DcfSample dcf_sample(const DcfGeo &g, float kx, float ky, float kz) {
  DcfSample t;
  const float kr = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz)));
  t.sc = (float)((double)kr / 128.0 * (double)(g.acc - 1.0f) + 1.0);
  const float k[3] = {kx, ky, kz};
  t.ok = true;
  for (int d = 0; d < 3; d++) {
    const float c = (float)(g.S[d] / 2);
    t.dk[d] = __fadd_rn(__fmul_rn(k[d], g.og), c);
    const float w = __fmul_rn(t.sc, g.dwin);
    t.s[d] = max((int)ceilf(__fsub_rn(t.dk[d], w)), 0);
    t.e[d] = min((int)floorf(__fadd_rn(t.dk[d], w)), g.S[d] - 1);
    if (t.s[d] >= g.S[d] || t.e[d] < 0) t.ok = false;
  }
  return t;
}

// lut((int)del)*(1.0 - d) + lut((int)del + 1)*d, del = |600 (dk - l)| / s
__device__ __forceinline__ double dcf_axis_weight(const float *lut, float dk, int l, float sc) {
  const float del = __fdiv_rn(fabsf(__fmul_rn(600.0f, __fsub_rn(dk, (float)l))), sc);
  const int i = (int)del;
  const float d = __fsub_rn(del, (float)i);
  return (double)lut[i] * (1.0 - (double)d) + (double)lut[i + 1] * (double)d;
}

constexpr int DCF_MAX_TAPS = 16;  // per axis; the plan rejects kernels wider than this

__device__ __forceinline__ void dcf_axis_weights(const DcfGeo &g, const DcfSample &t, int d, double *w) {
  const int n = t.e[d] - t.s[d] + 1;
  for (int a = 0; a < n && a < DCF_MAX_TAPS; a++) w[a] = dcf_axis_weight(g.lut, t.dk[d], t.s[d] + a, t.sc);
}

__global__ void k_dcf_grid(DcfGeo g, int64_t M, const float *__restrict__ kx, const float *__restrict__ ky,
                           const float *__restrict__ kz, const float *__restrict__ kw, float *X) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = kw[i];
    if (v == 0.0f) continue;  // src/DCFgridFFT.cpp:199
    const DcfSample t = dcf_sample(g, kx[i], ky[i], kz[i]);
    if (!t.ok) continue;
    double wx[DCF_MAX_TAPS], wy[DCF_MAX_TAPS], wz[DCF_MAX_TAPS];
    dcf_axis_weights(g, t, 0, wx);
    dcf_axis_weights(g, t, 1, wy);
    dcf_axis_weights(g, t, 2, wz);
    for (int lz = t.s[2]; lz <= t.e[2]; lz++) {
      const float wtz = (float)wz[lz - t.s[2]];
      for (int ly = t.s[1]; ly <= t.e[1]; ly++) {
        const float wty = (float)((double)wtz * wy[ly - t.s[1]]);
        float *row = X + ((int64_t)lz * g.S[1] + ly) * g.S[0];
        for (int lx = t.s[0]; lx <= t.e[0]; lx++) {
          const float wtx = (float)((double)wty * wx[lx - t.s[0]]);
          atomicAdd(row + lx, __fmul_rn(wtx, v));
        }
      }
    }
  }
}

__global__ void k_dcf_degrid(DcfGeo g, int64_t M, const float *__restrict__ kx, const float *__restrict__ ky,
                             const float *__restrict__ kz, const float *__restrict__ X, float *kw2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const DcfSample t = dcf_sample(g, kx[i], ky[i], kz[i]);
    float acc = 0.0f;
    if (t.ok) {
      double wx[DCF_MAX_TAPS], wy[DCF_MAX_TAPS], wz[DCF_MAX_TAPS];
      dcf_axis_weights(g, t, 0, wx);
      dcf_axis_weights(g, t, 1, wy);
      dcf_axis_weights(g, t, 2, wz);
      for (int lz = t.s[2]; lz <= t.e[2]; lz++) {
        const float wtz = (float)wz[lz - t.s[2]];
        for (int ly = t.s[1]; ly <= t.e[1]; ly++) {
          const float wty = (float)((double)wtz * wy[ly - t.s[1]]);
          const float *row = X + ((int64_t)lz * g.S[1] + ly) * g.S[0];
          for (int lx = t.s[0]; lx <= t.e[0]; lx++) {
            const float wtx = (float)((double)wty * wx[lx - t.s[0]]);
            acc = __fadd_rn(acc, __fmul_rn(wtx, __ldg(row + lx)));
          }
        }
      }
    }
    kw2[i] = acc;
  }
}

__global__ void k_dcf_update(int64_t M, float *kw, const float *__restrict__ kw2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = kw2[i];
    kw[i] = (fabsf(d) < 1e-3f) ? 0.0f : __fdiv_rn(kw[i], d);
  }
}

__global__ void k_dcf_final(DcfGeo g, int64_t M, const float *__restrict__ kx, const float *__restrict__ ky,
                            const float *__restrict__ kz, float *kw) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const DcfSample t = dcf_sample(g, kx[i], ky[i], kz[i]);
    const double s = (double)t.sc;
    kw[i] = fabsf((float)((double)kw[i] * (s * s * s)));
  }
}

__global__ void k_dcf_fill(int64_t M, float v, float *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = v;
}

__global__ void k_dcf_scale_traj(int64_t M, const float *__restrict__ in, float s, float *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __fmul_rn(in[i], s);
}

}  // namespace

// Polynomial kernel table of DCFgridFFT (loadKernelTable / loadKernelTable2,
// src/DCFgridFFT.cpp:47-84), length (int)(dwin*600) + 100, normalised to sum 0.5*600.
void dcf_table(float dwin, int kernel, std::vector<float> &t) {
  const int len = (int)((float)dwin * 600.0f) + 100;
  t.assign(len, 0.0f);
  static const double c[2][6] = {{1., 0.04522831, -3.36020304, 1.12417012, 2.82448025, -1.63447764},
                                 {1., 0.03056504, -3.01961845, 0.6679865, 2.77924058, -1.45923643}};
  const double *k = c[kernel ? 1 : 0];
  for (int i = 0; i < len; i++) {
    const double x = double(i) / double(len), x2 = x * x, x4 = x2 * x2, x3 = x * x2, x5 = x * x4;
    t[i] = (float)(k[0] + k[1] * x + k[2] * x2 + k[3] * x3 + k[4] * x4 + k[5] * x5);
  }
  double sum = 0;
  for (int i = 0; i < len; i++) sum += t[i];
  const double f = 0.5 * 600.0f / sum;
  for (int i = 0; i < len; i++) t[i] = (float)(t[i] * f);
}

// kx/ky/kz: device arrays of M samples; kw: device output.
mrg_status dcf_pipe(const float *kx, const float *ky, const float *kz, int64_t M, const int N[3], int iters,
                    float dwin, float scale, float overgrid, float acc, int kernel, float *kw, cudaStream_t st) {
  DcfGeo g;
  // RECON::dcf_calc allocates its image as (overgrid Nz + 16, overgrid Ny + 16, overgrid Nx
  // + 16) in column-major order (src/recon_lib.cpp:873-875) and DCFgridFFT takes the first
  // extent as Sx (src/DCFgridFFT.cpp:174-176, :325-327): x and z extents are swapped, which
  // matters for anisotropic matrices only
  for (int d = 0; d < 3; d++) g.S[d] = (int)(overgrid * N[2 - d] + 16);
  g.og = overgrid;
  g.dwin = dwin;
  g.acc = acc;
  // widest kernel: s at |k| = the grid's half extent
  const double kmax = 0.5 * std::max(g.S[0], std::max(g.S[1], g.S[2])) / overgrid * std::sqrt(3.0);
  const double smax = kmax / 128.0 * std::fabs(acc - 1.0) + 1.0;
  if (2 * smax * dwin + 2 > DCF_MAX_TAPS) {
    set_error("density-compensation kernel wider than this build's tap limit");
    return MRG_ERR_UNSUPPORTED;
  }
  std::vector<float> lut;
  dcf_table(dwin, kernel, lut);
  const int64_t S3 = (int64_t)g.S[0] * g.S[1] * g.S[2];
  float *dl = nullptr, *X = nullptr, *kw2 = nullptr, *sk = nullptr;
  mrg_status rs = MRG_OK;
  auto fail = [&](mrg_status e) {
    cudaFree(dl);
    cudaFree(X);
    cudaFree(kw2);
    cudaFree(sk);
    return e;
  };
  if (cudaMalloc(&dl, sizeof(float) * (lut.size() + 2)) != cudaSuccess ||
      cudaMalloc(&X, sizeof(float) * S3) != cudaSuccess || cudaMalloc(&kw2, sizeof(float) * M) != cudaSuccess ||
      cudaMalloc(&sk, sizeof(float) * 3 * M) != cudaSuccess) {
    cudaGetLastError();
    set_error("device allocation failed (density compensation)");
    return fail(MRG_ERR_NOMEM);
  }
  lut.push_back(0.0f);
  lut.push_back(0.0f);  // del < len - 2 always; padding for the +1 read
  if (cudaMemcpyAsync(dl, lut.data(), sizeof(float) * lut.size(), cudaMemcpyHostToDevice, st) != cudaSuccess) {
    set_error("copy of the kernel table failed");
    return fail(MRG_ERR_CUDA);
  }
  g.lut = dl;
  const int nb = grid_blocks(M, 256);
  // k *= dcf_scale (src/recon_lib.cpp:880-882)
  float *skx = sk, *sky = sk + M, *skz = sk + 2 * M;
  k_dcf_scale_traj<<<nb, 256, 0, st>>>(M, kx, scale, skx);
  k_dcf_scale_traj<<<nb, 256, 0, st>>>(M, ky, scale, sky);
  k_dcf_scale_traj<<<nb, 256, 0, st>>>(M, kz, scale, skz);
  k_dcf_fill<<<nb, 256, 0, st>>>(M, 1.0f, kw);  // Kweight = 1
  for (int k = 0; k < 4; k++) count_launch();
  for (int it = 0; it < iters; it++) {
    if ((rs = launch_zero(X, sizeof(float) * S3, st)) != MRG_OK) return fail(rs);
    k_dcf_grid<<<nb, 256, 0, st>>>(g, M, skx, sky, skz, kw, X);
    count_launch();
    k_dcf_degrid<<<nb, 256, 0, st>>>(g, M, skx, sky, skz, X, kw2);
    count_launch();
    k_dcf_update<<<nb, 256, 0, st>>>(M, kw, kw2);
    count_launch();
  }
  k_dcf_final<<<nb, 256, 0, st>>>(g, M, skx, sky, skz, kw);
  count_launch();
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
    set_error(std::string("density compensation: ") + cudaGetErrorString(cudaGetLastError()));
    return fail(MRG_ERR_CUDA);
  }
  fail(MRG_OK);
  return MRG_OK;
}

}  // namespace mrg
