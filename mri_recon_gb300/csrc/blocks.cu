// Standalone C ABI for the FISTA and CLEAR building blocks: wavelet, fraction / soft
// threshold and the low-rank block operations (time and coil), on caller buffers.
#include <cstring>

#include "mrg_internal.h"

using namespace mrg;

namespace {
struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { cudaFree(p); }
};

bool is_dev(const void *ptr) {
  cudaPointerAttributes a;
  if (!ptr || cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device view of a caller buffer (host buffers copied in; written back by the caller).
mrg_status view(const void *ptr, size_t bytes, DevBuf &tmp, cudaStream_t st, float2 **out) {
  if (is_dev(ptr)) {
    *out = (float2 *)const_cast<void *>(ptr);
    return MRG_OK;
  }
  MRG_CUDA(cudaMalloc(&tmp.p, bytes));
  MRG_CUDA(cudaMemcpyAsync(tmp.p, ptr, bytes, cudaMemcpyHostToDevice, st));
  *out = (float2 *)tmp.p;
  return MRG_OK;
}

mrg_status back(void *ptr, const DevBuf &tmp, size_t bytes, cudaStream_t st) {
  if (tmp.p) {
    MRG_CUDA(cudaMemcpyAsync(ptr, tmp.p, bytes, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return MRG_OK;
}
}  // namespace

extern "C" {

mrg_status mrg_wavelet(void *X, int nvol, int Nx, int Ny, int Nz, const int levels[3], const int shift[3], int wave_type,
                       int inverse, void *stream) {
  if (!X || !levels || !shift || nvol <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || wave_type < 0 || wave_type > 1) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  int L[3], ml;
  wavelet_levels(N, levels, L, &ml);
  int sh[3];
  for (int d = 0; d < 3; d++) {
    if (shift[d] < 0) {
      set_error("wavelet shifts must be non-negative (rand() % wN in the reference)");
      return MRG_ERR_INVALID;
    }
    sh[d] = shift[d];
  }
  const size_t bytes = sizeof(float2) * (size_t)nvol * Nx * Ny * Nz;
  DevBuf tmp, dsh;
  float2 *d;
  MRG_TRY(view(X, bytes, tmp, st, &d));
  MRG_CUDA(cudaMalloc(&dsh.p, sizeof(sh)));
  MRG_CUDA(cudaMemcpyAsync(dsh.p, sh, sizeof(sh), cudaMemcpyHostToDevice, st));
  MRG_TRY(wavelet3d(d, nvol, N, L, ml, (const int *)dsh.p, wave_type, inverse, st));
  MRG_TRY(back(X, tmp, bytes, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

mrg_status mrg_fraction_threshold(const void *X, int nvol, int64_t nvox, float fraction, float *value, void *stream) {
  if (!X || !value || nvol <= 0 || nvox <= 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = (int64_t)nvol * nvox;
  DevBuf tmp, out;
  float2 *d;
  MRG_TRY(view(X, sizeof(float2) * n, tmp, st, &d));
  ThrWork w;
  mrg_status s = thr_alloc(w, n);
  if (s == MRG_OK) {
    MRG_CUDA(cudaMalloc(&out.p, sizeof(float)));
    s = fraction_threshold(d, n, fraction, 1.0f, w, (float *)out.p, st);
    if (s == MRG_OK && cudaMemcpyAsync(value, out.p, sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess) s = MRG_ERR_CUDA;
    if (s == MRG_OK && cudaStreamSynchronize(st) != cudaSuccess) s = MRG_ERR_CUDA;
  }
  thr_free(w);
  return s;
}

mrg_status mrg_soft_threshold(void *X, int64_t n, float value, void *stream) {
  if (!X || n <= 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf tmp, dv;
  float2 *d;
  MRG_TRY(view(X, sizeof(float2) * n, tmp, st, &d));
  MRG_CUDA(cudaMalloc(&dv.p, sizeof(float)));
  MRG_CUDA(cudaMemcpyAsync(dv.p, &value, sizeof(float), cudaMemcpyHostToDevice, st));
  MRG_TRY(soft_threshold(d, n, (const float *)dv.p, st));
  MRG_TRY(back(X, tmp, sizeof(float2) * n, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

mrg_status mrg_llr_update_threshold(const void *X, int nframes, int Nx, int Ny, int Nz, const int block[3],
                                    float clear_amp, float clear_t2, int iteration, float *smax, void *stream) {
  if (!X || !block || !smax || nframes <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || block[0] < 1 || block[1] < 1 ||
      block[2] < 1) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  const size_t bytes = sizeof(float2) * (size_t)nframes * Nx * Ny * Nz;
  DevBuf tmp;
  float2 *d;
  MRG_TRY(view(X, bytes, tmp, st, &d));
  LlrWork w;
  mrg_status s = llr_update_ex(d, nframes, N, block, clear_amp, clear_t2, nullptr, iteration, w, st);
  if (s == MRG_OK && cudaMemcpyAsync(smax, w.smax, sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess) s = MRG_ERR_CUDA;
  if (s == MRG_OK && cudaStreamSynchronize(st) != cudaSuccess) s = MRG_ERR_CUDA;
  llr_free(w);
  return s;
}

mrg_status mrg_llr_thresh(void *X, int nframes, int Nx, int Ny, int Nz, const int block[3], int block_iter, float alpha,
                          float smax, int64_t rand_skip, void *stream) {
  if (!X || !block || nframes <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || block_iter <= 0 || rand_skip < 0 ||
      block[0] < 1 || block[1] < 1 || block[2] < 1) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  int bs[3];
  for (int d = 0; d < 3; d++) bs[d] = std::min(block[d], N[d]);
  // block shifts in the reference's draw order (clear.cpp:408-415)
  GlibcRand r;
  r.skip(rand_skip);
  std::vector<int> sh(3 * block_iter);
  for (int it = 0; it < block_iter; it++) {
    for (int d = 0; d < 3; d++) sh[3 * it + d] = r.next() % bs[d] - bs[d] / 2;
    if (block_iter == 1) sh[0] = sh[1] = sh[2] = 0;
  }
  const size_t bytes = sizeof(float2) * (size_t)nframes * Nx * Ny * Nz;
  DevBuf tmp, dsh, dsm;
  float2 *d;
  MRG_TRY(view(X, bytes, tmp, st, &d));
  MRG_CUDA(cudaMalloc(&dsh.p, sizeof(int) * sh.size()));
  MRG_CUDA(cudaMemcpyAsync(dsh.p, sh.data(), sizeof(int) * sh.size(), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaMalloc(&dsm.p, sizeof(float)));
  MRG_CUDA(cudaMemcpyAsync(dsm.p, &smax, sizeof(float), cudaMemcpyHostToDevice, st));
  MRG_TRY(llr_apply(d, nframes, N, bs, block_iter, alpha, (const int *)dsh.p, (const float *)dsm.p, st));
  MRG_TRY(back(X, tmp, bytes, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

static bool clear_args_ok(const void *X, int nframes, int ncoil, int Nx, int Ny, int Nz, const int block[3]) {
  if (!X || !block || nframes <= 0 || ncoil <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || block[0] < 1 || block[1] < 1 ||
      block[2] < 1) {
    set_error("bad argument");
    return false;
  }
  return true;
}

mrg_status mrg_clear_update_threshold(const void *X, int nframes, int ncoil, int Nx, int Ny, int Nz,
                                      const int block[3], float clear_amp, float clear_t2, int iteration,
                                      float *smax, void *stream) {
  if (!clear_args_ok(X, nframes, ncoil, Nx, Ny, Nz, block) || !smax) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  const int64_t nb64 = coil_llr_blocks(N, block);
  if (nb64 > (int64_t)(1 << 30)) {
    set_error("too many coil low-rank blocks (" + std::to_string(nb64) + ")");
    return MRG_ERR_UNSUPPORTED;
  }
  const int nb = (int)nb64;
  int np2 = 1;
  while (np2 < nb) np2 <<= 1;
  const size_t bytes = sizeof(float2) * (size_t)nframes * Nx * Ny * Nz * ncoil;
  DevBuf tmp, work;
  float2 *d;
  MRG_TRY(view(X, bytes, tmp, st, &d));
  MRG_CUDA(cudaMalloc(&work.p, sizeof(double) * (size_t)(nb + np2) + 16));
  double *sig = (double *)work.p;
  float *dsm = (float *)(sig + nb + np2);
  MRG_TRY(coil_llr_update(d, nframes, ncoil, N, block, clear_amp, clear_t2, iteration, sig, sig + nb, dsm, st));
  MRG_CUDA(cudaMemcpyAsync(smax, dsm, sizeof(float), cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

mrg_status mrg_clear_thresh(void *X, int nframes, int ncoil, int Nx, int Ny, int Nz, const int block[3],
                            int block_iter, float alpha, float smax, int64_t rand_skip, void *stream) {
  if (!clear_args_ok(X, nframes, ncoil, Nx, Ny, Nz, block) || block_iter <= 0 || rand_skip < 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  int bs[3];
  for (int d = 0; d < 3; d++) bs[d] = std::min(block[d], N[d]);
  // block shifts in the reference's draw order (clear.cpp:612-615); no zero-shift rule
  // for block_iter == 1 here, unlike the time low-rank threshold
  GlibcRand r;
  r.skip(rand_skip);
  std::vector<int> sh(3 * block_iter);
  for (int it = 0; it < block_iter; it++)
    for (int d = 0; d < 3; d++) sh[3 * it + d] = r.next() % bs[d] - bs[d] / 2;
  const size_t bytes = sizeof(float2) * (size_t)nframes * Nx * Ny * Nz * ncoil;
  DevBuf tmp, dsh, dsm;
  float2 *d;
  MRG_TRY(view(X, bytes, tmp, st, &d));
  MRG_CUDA(cudaMalloc(&dsh.p, sizeof(int) * sh.size()));
  MRG_CUDA(cudaMemcpyAsync(dsh.p, sh.data(), sizeof(int) * sh.size(), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaMalloc(&dsm.p, sizeof(float)));
  MRG_CUDA(cudaMemcpyAsync(dsm.p, &smax, sizeof(float), cudaMemcpyHostToDevice, st));
  MRG_TRY(coil_llr_thresh(d, nframes, ncoil, N, bs, alpha, block_iter, (const int *)dsh.p, (const float *)dsm.p, st));
  MRG_TRY(back(X, tmp, bytes, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

mrg_status mrg_clear_combine(const void *X, int nframes, int ncoil, int Nx, int Ny, int Nz, const int block[3],
                             void *out, void *stream) {
  if (!clear_args_ok(X, nframes, ncoil, Nx, Ny, Nz, block) || !out) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  const size_t nv = (size_t)nframes * Nx * Ny * Nz;
  DevBuf tmp, tout;
  float2 *d, *o;
  MRG_TRY(view(X, sizeof(float2) * nv * ncoil, tmp, st, &d));
  MRG_TRY(view(out, sizeof(float2) * nv, tout, st, &o));  // voxels outside whole blocks keep their values
  MRG_TRY(coil_combine(d, nframes, ncoil, N, block, o, st));
  MRG_TRY(back(out, tout, sizeof(float2) * nv, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

void mrg_espirit_params_default(mrg_espirit_params *p) {
  if (!p) return;
  for (int d = 0; d < 3; d++) {  // src/spirit.cpp:9-34
    p->kernel_radius[d] = 3.0f;
    p->calib_radius[d] = 12;
  }
  p->svd_thresh = 0.01f;
  p->square = 0;
}

mrg_status mrg_espirit(const void *images, int ncoil, int Nx, int Ny, int Nz, const mrg_espirit_params *params,
                       void *maps, int *kept, double *sv, int sv_cap, void *stream) {
  if (!images || !maps || !params || ncoil <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || (sv && sv_cap < 0)) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  for (int d = 0; d < 3; d++)
    if (!(params->kernel_radius[d] >= 0.0f) || params->kernel_radius[d] > 7.0f) {
      set_error("ESPIRiT kernel radius must be in [0, 7]");
      return MRG_ERR_INVALID;
    }
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  const size_t bytes = sizeof(float2) * (size_t)Nx * Ny * Nz * ncoil;
  DevBuf ti, tm;
  float2 *di, *dm;
  MRG_TRY(view(images, bytes, ti, st, &di));
  MRG_TRY(view(maps, bytes, tm, st, &dm));
  EspiritParams q;
  for (int d = 0; d < 3; d++) {
    q.kr_f[d] = params->kernel_radius[d];
    q.cr[d] = params->calib_radius[d];
  }
  q.svd_thresh = params->svd_thresh;
  q.square = params->square;
  q.sv_out = sv;
  q.sv_cap = sv ? sv_cap : 0;
  MRG_TRY(espirit_maps(di, ncoil, N, q, dm, kept, st));
  MRG_TRY(back(maps, tm, bytes, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

mrg_status mrg_gaussian_blur(void *X, int nvol, int Nx, int Ny, int Nz, int64_t vol_stride, const float sigma[3],
                             void *stream) {
  if (!X || !sigma || nvol <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  const int64_t nimg = (int64_t)Nx * Ny * Nz;
  if (nvol > 1 && vol_stride < nimg) {
    set_error("vol_stride smaller than one volume");
    return MRG_ERR_INVALID;
  }
  const int64_t vs = nvol > 1 ? vol_stride : nimg;
  cudaStream_t st = (cudaStream_t)stream;
  const int N[3] = {Nx, Ny, Nz};
  const size_t bytes = sizeof(float2) * (size_t)(vs * (nvol - 1) + nimg);
  DevBuf tmp;
  float2 *d;
  MRG_TRY(view(X, bytes, tmp, st, &d));
  MRG_TRY(gaussian_blur_ex(d, nvol, N, 1, vs, sigma, st));
  return back(X, tmp, bytes, st);
}

mrg_status mrg_sos_normalize(void *maps, int ncoil, int64_t coil_stride, int64_t nvox, void *stream) {
  if (!maps || ncoil <= 0 || nvox <= 0 || (ncoil > 1 && coil_stride < nvox)) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  const int64_t vs = ncoil > 1 ? coil_stride : nvox;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = sizeof(float2) * (size_t)(vs * (ncoil - 1) + nvox);
  DevBuf tmp;
  float2 *d;
  MRG_TRY(view(maps, bytes, tmp, st, &d));
  MRG_TRY(sos_normalize_ex(d, ncoil, nvox, 1, vs, st));
  return back(maps, tmp, bytes, st);
}

void mrg_dcf_params_default(mrg_dcf_params *q) {
  if (!q) return;
  q->iters = 20;       // -dcf_iter      (src/recon_lib.cpp:126)
  q->dwin = 2.1f;      // -dcf_dwin      (:127)
  q->scale = 1.0f;     // -dcf_scale     (:128)
  q->overgrid = 2.1f;  // -dcf_overgrid  (:129)
  q->acc = 1.0f;       // -dcf_acc       (:130)
  q->kernel = 0;       // DCFgridFFT::POLY_KERNEL (:857)
}

mrg_status mrg_dcf_pipe(const float *kx, const float *ky, const float *kz, int64_t M, int Nx, int Ny, int Nz,
                        const mrg_dcf_params *q_in, float *kw, void *stream) {
  if (!kx || !ky || !kz || !kw || M <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || Nx > 65536 || Ny > 65536 || Nz > 65536) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  mrg_dcf_params q;
  if (q_in) q = *q_in; else mrg_dcf_params_default(&q);
  // bounded so that the grid, (int)(overgrid N + 16) per axis, and the kernel table stay small
  if (q.iters < 0 || !(q.dwin > 0 && q.dwin <= 16) || !(q.scale > 0) || !(q.overgrid > 0 && q.overgrid <= 8) ||
      !(q.acc > 0) || q.kernel < 0 || q.kernel > 1) {
    set_error("bad density-compensation parameters");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = sizeof(float) * (size_t)M;
  DevBuf tx, ty, tz, tw;
  float2 *dx, *dy, *dz, *dw;
  MRG_TRY(view(kx, bytes, tx, st, &dx));
  MRG_TRY(view(ky, bytes, ty, st, &dy));
  MRG_TRY(view(kz, bytes, tz, st, &dz));
  MRG_TRY(view(kw, bytes, tw, st, &dw));
  const int N[3] = {Nx, Ny, Nz};
  MRG_TRY(dcf_pipe((const float *)dx, (const float *)dy, (const float *)dz, M, N, q.iters, q.dwin, q.scale,
                   q.overgrid, q.acc, q.kernel, (float *)dw, st));
  return back(kw, tw, bytes, st);
}

}  // extern "C"
