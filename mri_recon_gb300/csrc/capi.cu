// Plan object and C ABI (include/mrg.h).
//
// A plan owns the device state that one reference gridFFT / gridFFT_CoilThreaded
// instance owns on the host (k3d_grid, LUT, windows; src/gridFFT.h:28-194),
// plus the per-frame sorted trajectories and the CG / FISTA work vectors of
// RECON::full_recon (src/recon_lib.cpp:1523-2212).
//
// Device memory layout (complex64 unless noted):
//   grid  [Sz][Sy][Sx][C]        oversampled k-space, all coils adjacent
//   t2    [Sz][Sy][Nx][C]        after the y pass (E) / before the y pass (E^H)
//   t1    [Sz][Ny][Nx][C]        after the z pass (E) / before the z pass (E^H)
//   smap  [Nz][Ny][Nx][C]        coil maps, coils adjacent
//   y     [nvalid][C]            k-space samples in tile-sorted order
//   images [frame][Nz][Ny][Nx]   as the reference's X, R, P, LHS
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>

#include "mrg_internal.h"

namespace mrg {
static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
std::atomic<int64_t> g_launches{0};

int device_sms() {
  static std::mutex mu;
  static int sms[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 152;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!sms[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
      cudaGetLastError();
      n = 152;
    }
    sms[dev] = n;
  }
  return sms[dev];
}
}  // namespace mrg

using namespace mrg;

struct mrg_plan {
  Geometry geo;
  mrg_config cfg;
  int C = 1, T = 1;
  int64_t nimg = 0;
  int B = 8;
  int max_pairs = 4096;
  float *d_lut = nullptr, *d_win = nullptr;
  float2 *d_grid = nullptr, *d_t2 = nullptr, *d_t1 = nullptr, *d_smap = nullptr;
  bool has_smaps = false;
  float2 *d_y = nullptr;
  int64_t y_cap = 0;
  std::vector<FrameTraj> frames;
  // solver state
  float2 *d_R = nullptr, *d_P = nullptr, *d_L = nullptr, *d_Xo = nullptr;
  double *d_part = nullptr;
  int nblk = 0;
  Scalars *d_sc = nullptr;
  double *d_resid = nullptr;
  int resid_cap = 0;
  // staging for host pointers
  void *d_stage[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t stage_cap[4] = {0, 0, 0, 0};
  float timings[8] = {0};
  int timing_on = 0, timing_calls = 0;
  int fft_ib[6] = {0, 0, 0, 0, 0, 0};  // lines per CTA per FFT pass (0: default)
  int fft_xp[6] = {0, 0, 0, 0, 0, 0};  // persistent set_image / accumulate kernel per pass
  bool fft_tuned = false;
  cudaEvent_t tev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int64_t graph_kernels = 0;  // kernels per replay of cg_exec
  // cached CG graph
  cudaGraphExec_t cg_exec = nullptr;
  void *cg_key[2] = {nullptr, nullptr};
  // autotuned launch shapes, reused while the sample count stays within 2x
  bool tuned = false;
  int tuned_G = 0, tuned_spb = 0, tuned_cpl = 0, tuned_uy = 0, tuned_cc = 0;
  int64_t tuned_nvalid = 0;
  float tuned_ms[2] = {0.f, 0.f};
  // FISTA state
  ThrWork thr;
  LlrWork llr;
  int *d_wshift = nullptr, *d_lshift = nullptr;
  float *d_thr = nullptr;
  // bounded device-side waits: limit of one wait and the error word the kernels set
  long long wait_ns = MRG_DEFAULT_WAIT_NS;
  int *d_err = nullptr;
  int last_iters = 0;  // iterations the last mrg_cg / mrg_fista / mrg_clear ran
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
static GridConst grid_const(const mrg_plan *p) {
  GridConst g;
  for (int d = 0; d < 3; d++) {
    g.S[d] = p->geo.S[d];
    g.grid[d] = p->geo.grid[d];
    g.cen[d] = (float)(p->geo.S[d] / 2);
    g.dwin[d] = p->geo.dwin[d];
    g.gmod[d] = p->geo.grid_mod[d];
    g.lut[d] = p->d_lut + (size_t)d * p->geo.lut_len;
    g.nt[d] = p->geo.S[d] / p->B;
  }
  g.nb[0] = p->geo.S[0] / BLK_X;
  g.nb[1] = p->geo.S[1] / BLK_Y;
  g.nb[2] = p->geo.S[2] / BLK_Z;
  g.k_rad = p->geo.k_rad;
  g.B = p->B;
  g.mbits = 0;
  while ((1 << g.mbits) < std::max(g.nt[0], std::max(g.nt[1], g.nt[2]))) g.mbits++;
  g.C = p->C;
  g.eval = p->cfg.kernel_eval;
  g.grid_mode = p->cfg.grid_mode;
  for (int d = 0; d < 3; d++) {
    g.beta[d] = p->geo.beta[d];
    g.kb_norm[d] = p->geo.kb_norm[d];
  }
  g.err = p->d_err;
  g.wait_ns = p->wait_ns;
  return g;
}

// After the caller's stream has been synchronised: MRG_ERR_TIMEOUT (and the word cleared)
// when a bounded device-side wait of this plan's kernels ran out since the last check.
static mrg_status plan_check(mrg_plan *p, cudaStream_t st) {
  if (!p->d_err) return MRG_OK;
  int h = 0;
  MRG_CUDA(cudaMemcpyAsync(&h, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  if (h) {
    MRG_CUDA(cudaMemsetAsync(p->d_err, 0, sizeof(int), st));
    MRG_CUDA(cudaStreamSynchronize(st));
    if (h == MRG_REGION_RANGE) {
      set_error("tensor-core gridding met a work item outside the grid and skipped it; results of the calls "
                "since the last check are incomplete");
      return MRG_ERR_CUDA;
    }
    set_error("a bounded device-side wait ran out (tensor-core gridding gave up); results of the calls since "
              "the last check are incomplete");
    return MRG_ERR_TIMEOUT;
  }
  return MRG_OK;
}

// The reference's early-stop rule (src/recon_lib.cpp:2081-2087, :2154-2163): residual
// ratios of the last `range` iterations, their standard deviation in the reference's
// float / double mix, below `thresh`.
static bool early_stop_met(std::vector<float> &diffs, float ratio, int range, float thresh) {
  diffs.push_back(ratio);
  if ((int)diffs.size() > range) diffs.erase(diffs.begin());
  if ((int)diffs.size() != range) return false;
  double sum = 0.0, sq = 0.0;  // std::accumulate / std::inner_product with a double 0.0
  for (float v : diffs) {
    sum += v;
    sq += (double)v * v;
  }
  const float mean = (float)(sum / diffs.size());
  const float sq_sum = (float)sq;
  const float stdev = std::sqrt(sq_sum / (float)diffs.size() - mean * mean);
  return stdev < thresh;
}

static bool is_device_ptr(const void *ptr) {
  if (!ptr) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static mrg_status stage_buf(mrg_plan *p, int slot, size_t bytes, void **out) {
  if (p->stage_cap[slot] < bytes) {
    cudaFree(p->d_stage[slot]);
    p->d_stage[slot] = nullptr;
    p->stage_cap[slot] = 0;
    MRG_CUDA(cudaMalloc(&p->d_stage[slot], bytes));
    p->stage_cap[slot] = bytes;
  }
  *out = p->d_stage[slot];
  return MRG_OK;
}

// Device view of a caller buffer: device pointers pass through, host buffers are
// copied into staging slot `slot` (when `copy_in`).
static mrg_status dev_view(mrg_plan *p, int slot, const void *ptr, size_t bytes, bool copy_in, cudaStream_t st,
                           void **dev, bool *staged) {
  *staged = false;
  if (!ptr) {
    *dev = nullptr;
    return MRG_OK;
  }
  if (is_device_ptr(ptr)) {
    *dev = const_cast<void *>(ptr);
    return MRG_OK;
  }
  MRG_TRY(stage_buf(p, slot, bytes, dev));
  if (copy_in) {
    // large pinned inputs are read by the SMs through the buffer's device-side alias
    // (both ends of the range pinned and mapped contiguously, so every read stays inside it)
    cudaPointerAttributes a, z;
    const char *last = static_cast<const char *>(ptr) + bytes - 1;
    const bool pinned = bytes >= ((size_t)64 << 20) && cudaPointerGetAttributes(&a, ptr) == cudaSuccess &&
                        a.type == cudaMemoryTypeHost && a.devicePointer && ((uintptr_t)a.devicePointer & 15) == 0 &&
                        cudaPointerGetAttributes(&z, last) == cudaSuccess && z.type == cudaMemoryTypeHost &&
                        static_cast<const char *>(z.devicePointer) == static_cast<const char *>(a.devicePointer) + (bytes - 1);
    if (!pinned) cudaGetLastError();
    if (pinned) MRG_TRY(launch_copy_from_host(*dev, a.devicePointer, bytes, st));
    else MRG_CUDA(cudaMemcpyAsync(*dev, ptr, bytes, cudaMemcpyHostToDevice, st));
  }
  *staged = true;
  return MRG_OK;
}

// A captured CG graph holds raw pointers: drop it whenever a buffer it uses moves.
static void invalidate_graphs(mrg_plan *p) {
  if (p->cg_exec) {
    cudaGraphExecDestroy(p->cg_exec);
    p->cg_exec = nullptr;
  }
}

static mrg_status ensure_y(mrg_plan *p, int64_t n) {
  if (p->y_cap >= n) return MRG_OK;
  invalidate_graphs(p);
  cudaFree(p->d_y);
  p->d_y = nullptr;
  p->y_cap = 0;
  MRG_CUDA(cudaMalloc(&p->d_y, sizeof(float2) * (size_t)std::max<int64_t>(n, 1)));
  p->y_cap = n;
  return MRG_OK;
}

// Default lines per CTA of a pass of length S: a multiple of C up to the kernel's limit
// (32, or 16 for lines above 384 points).
static int pass_ib(int64_t inner, int C, int S) {
  const int m = fft_max_lines_per_cta(S);
  if (C > m) return m;
  return C * (m / C);
}

// Lines per CTA of FFT pass k (0-2: E z/y/x, 3-5: E^H x/y/z): the autotuned value
// when it is valid for this pass, else the default (a multiple of C, up to 32).
static int plan_ib(const mrg_plan *p, int k, int64_t inner, int C, bool accum, int S) {
  const int def = pass_ib(inner, C, S);
  const int v = p->fft_ib[k];
  if (v <= 0 || v == def || v > fft_max_lines_per_cta(S)) return def;
  if (accum && (v % C) != 0) return def;  // the coil sum must stay inside a CTA
  if (v % 2) return def;
  return v;
}

// Scale of one FFT pass over S points: 1/sqrt(S), as gridFFT's fft3 scales each axis
// (src/ArrayTemplates.cpp:311, :338-342), or 1 for a plan with fft_norm = 1, whose
// transforms are unnormalised as gridFFT_CoilThreaded's FFTW calls are
// (src/gridFFT_CoilThreaded.cpp:570-893): its E and E^H are then sqrt(Sx Sy Sz) larger.
static float pass_scale(const mrg_plan *p, int64_t S) {
  return p->cfg.fft_norm ? 1.0f : (float)(1. / std::sqrt((float)S));
}

// Stage timing (mrg_set_timing): events between the four stages of E or E^H.
static void tmark(mrg_plan *p, int k, cudaStream_t st) {
  if (p->timing_on) cudaEventRecord(p->tev[k], st);
}
static void tcollect(mrg_plan *p, int base) {
  if (!p->timing_on) return;
  cudaEventSynchronize(p->tev[4]);
  for (int k = 0; k < 4; k++) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->tev[k], p->tev[k + 1]);
    p->timings[base + k] += ms;
  }
  if (base == 0) p->timing_calls += 1;
  if (p->cfg.time_grid) {
    const float *t = p->timings + base;
    const bool one = (p->C == 1);  // single-coil plans run the reference's pass order
    if (base == 0)
      printf(one ? "Backward::copy+zfft:%.3f,yfft:%.3f,xfft:%.3f,igrid:%.3f ms\n"
                 : "Backward::copy+xfft:%.3f,zfft:%.3f,yfft:%.3f,igrid:%.3f ms\n", t[0], t[1], t[2], t[3]);
    else
      printf(one ? "Forward::grid:%.3f,xfft:%.3f,yfft:%.3f,zfft+accumulate:%.3f ms\n"
                 : "Forward::grid:%.3f,yfft:%.3f,zfft:%.3f,xfft+accumulate:%.3f ms\n", t[0], t[1], t[2], t[3]);
  }
}

// E for one frame: image X -> sorted samples y (minus diff if given); with
// `weigh` the samples come out multiplied by kw and the taper, ready for run_EH.
// smap: interleaved plan maps when C > 1 or an explicit single-coil map (may be NULL).
static mrg_status run_E_grid(mrg_plan *p, const float2 *X, const float2 *smap, cudaStream_t st);

static mrg_status run_E(mrg_plan *p, const FrameTraj &ft, const float2 *X, const float2 *smap, const float2 *diff,
                        float2 *y, bool weigh, cudaStream_t st) {
  MRG_TRY(run_E_grid(p, X, smap, st));
  tmark(p, 3, st);
  // ungrid (src/gridFFT.cpp:1166-1322)
  const GridConst gc = grid_const(p);
  MRG_TRY(launch_ungrid(gc, ft, p->d_grid, diff, y, weigh, st));
  tmark(p, 4, st);
  tcollect(p, 0);
  return MRG_OK;
}

// E up to the oversampled grid: set_image + x FFT, z FFT, y FFT (src/gridFFT.cpp:645-671, :972-986).
// Single-coil plans keep the reference's pass order (E: z, y, x; E^H: x, y, z): with one
// coil the z lines of neighbouring x are adjacent in memory, so the image-side passes
// (set_image, accumulate) on z lines are coalesced.  With coils innermost it is the x lines
// that hold contiguous images and maps, so multi-coil plans run E as x, z, y and E^H as
// y, z, x (run_E_grid, run_EH_yz, run_EH, run_EH_crop further down).
static mrg_status run_E_grid_zxy(mrg_plan *p, const float2 *X, const float2 *smap, cudaStream_t st) {
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Nx = g.N[0], Ny = g.N[1], Nz = g.N[2], Sx = g.S[0], Sy = g.S[1], Sz = g.S[2];
  const float *wx = p->d_win, *wy = p->d_win + Sx, *wz = p->d_win + Sx + Sy;
  FftPass a;
  memset(&a, 0, sizeof(a));
  // z pass with set_image (src/gridFFT.cpp:972-986 + fft3 along z)
  a.S = (int)Sz; a.sign = -1; a.mode = FFT_SETIMG;
  a.Lin = (int)Nz; a.in_off = g.og[2]; a.Lout = (int)Sz; a.out_off = 0;
  a.inner = (int)(Nx * C); a.IB = plan_ib(p, 0, a.inner, C, false, a.S); a.lfast = 0;
  a.nlines = Ny * Nx * C;
  a.in_ls = Nx * Ny * C; a.in_os = Nx * C; a.out_ls = Ny * Nx * C; a.out_os = Nx * C;
  a.scale = pass_scale(p, Sz);
  a.in = smap; a.smap = smap; a.has_smap = smap != nullptr; a.X = X; a.out = p->d_t1;
  a.wl = wz + g.og[2]; a.wo = wy + g.og[1]; a.wi = wx + g.og[0]; a.C = C;
  tmark(p, 0, st);
  fft_vectorize(a);
  MRG_TRY(launch_fft(a, st));
  tmark(p, 1, st);
  // y pass
  FftPass b;
  memset(&b, 0, sizeof(b));
  b.S = (int)Sy; b.sign = -1; b.mode = FFT_PLAIN;
  b.Lin = (int)Ny; b.in_off = g.og[1]; b.Lout = (int)Sy; b.out_off = 0;
  b.inner = (int)(Nx * C); b.IB = plan_ib(p, 1, b.inner, C, false, b.S);
  b.nlines = Sz * Nx * C;
  b.in_ls = Nx * C; b.in_os = Ny * Nx * C; b.out_ls = Nx * C; b.out_os = Sy * Nx * C;
  b.scale = pass_scale(p, Sy);
  b.in = p->d_t1; b.out = p->d_t2; b.C = C;
  fft_vectorize(b);
  MRG_TRY(launch_fft(b, st));
  tmark(p, 2, st);
  // x pass
  FftPass c;
  memset(&c, 0, sizeof(c));
  c.S = (int)Sx; c.sign = -1; c.mode = FFT_PLAIN;
  c.Lin = (int)Nx; c.in_off = g.og[0]; c.Lout = (int)Sx; c.out_off = 0;
  c.inner = C; c.IB = (C == 1) ? pass_ib(C, C, c.S) : plan_ib(p, 2, C, C, false, c.S); c.lfast = (C == 1);
  c.nlines = Sz * Sy * C;
  c.in_ls = C; c.in_os = Nx * C; c.out_ls = C; c.out_os = Sx * C;
  c.scale = pass_scale(p, Sx);
  c.in = p->d_t2; c.out = p->d_grid; c.C = C;
  fft_vectorize(c);
  MRG_TRY(launch_fft(c, st));
  return MRG_OK;
}

// E^H for one frame: weighted sorted samples yw (data * kw * taper) -> X += ...
// E^H up to the y transform: grid, x and y inverse FFT passes; the result is in d_t1
// ([Sz][Ny][Nx][C], y and x already cropped).
static mrg_status run_EH_xy(mrg_plan *p, const FrameTraj &ft, const float2 *y, cudaStream_t st) {
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Nx = g.N[0], Ny = g.N[1], Sx = g.S[0], Sy = g.S[1], Sz = g.S[2];
  const GridConst gc = grid_const(p);
  tmark(p, 0, st);
  MRG_TRY(launch_grid(gc, ft, y, p->d_grid, st));  // src/gridFFT.cpp:1009-1164
  tmark(p, 1, st);
  FftPass a;
  memset(&a, 0, sizeof(a));
  a.S = (int)Sx; a.sign = +1; a.mode = FFT_PLAIN;
  a.Lin = (int)Sx; a.in_off = 0; a.Lout = (int)Nx; a.out_off = g.og[0];
  a.inner = C; a.IB = (C == 1) ? pass_ib(C, C, a.S) : plan_ib(p, 3, C, C, false, a.S); a.lfast = (C == 1);
  a.nlines = Sz * Sy * C;
  a.in_ls = C; a.in_os = Sx * C; a.out_ls = C; a.out_os = Nx * C;
  a.scale = pass_scale(p, Sx);
  a.in = p->d_grid; a.out = p->d_t2; a.C = C;
  fft_vectorize(a);
  MRG_TRY(launch_fft(a, st));
  tmark(p, 2, st);
  FftPass b;
  memset(&b, 0, sizeof(b));
  b.S = (int)Sy; b.sign = +1; b.mode = FFT_PLAIN;
  b.Lin = (int)Sy; b.in_off = 0; b.Lout = (int)Ny; b.out_off = g.og[1];
  b.inner = (int)(Nx * C); b.IB = plan_ib(p, 4, b.inner, C, false, b.S);
  b.nlines = Sz * Nx * C;
  b.in_ls = Nx * C; b.in_os = Sy * Nx * C; b.out_ls = Nx * C; b.out_os = Ny * Nx * C;
  b.scale = pass_scale(p, Sy);
  b.in = p->d_t2; b.out = p->d_t1; b.C = C;
  fft_vectorize(b);
  MRG_TRY(launch_fft(b, st));
  tmark(p, 3, st);
  return MRG_OK;
}

static mrg_status run_EH_xyz(mrg_plan *p, const FrameTraj &ft, const float2 *y, const float2 *smap, float2 *X,
                         cudaStream_t st) {
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Nx = g.N[0], Ny = g.N[1], Nz = g.N[2], Sx = g.S[0], Sy = g.S[1], Sz = g.S[2];
  const float *wx = p->d_win, *wy = p->d_win + Sx, *wz = p->d_win + Sx + Sy;
  MRG_TRY(run_EH_xy(p, ft, y, st));
  // z pass with accumulate (src/gridFFT.cpp:926-941)
  FftPass c;
  memset(&c, 0, sizeof(c));
  c.S = (int)Sz; c.sign = +1; c.mode = FFT_ACCUM;
  c.Lin = (int)Sz; c.in_off = 0; c.Lout = (int)Nz; c.out_off = g.og[2];
  c.inner = (int)(Nx * C); c.IB = plan_ib(p, 5, c.inner, C, true, c.S);
  c.nlines = Ny * Nx * C;
  c.in_ls = Ny * Nx * C; c.in_os = Nx * C; c.out_ls = Nx * Ny * C; c.out_os = Nx * C;
  c.scale = pass_scale(p, Sz);
  c.in = p->d_t1; c.smap = smap; c.has_smap = smap != nullptr; c.acc = X;
  c.acc_atomic = (c.IB % C) != 0; c.acc_l = Nx * Ny; c.acc_o = Nx;
  c.wl = wz + g.og[2]; c.wo = wy + g.og[1]; c.wi = wx + g.og[0]; c.C = C;
  fft_vectorize(c);
  MRG_TRY(launch_fft(c, st));
  tmark(p, 4, st);
  tcollect(p, 4);
  return MRG_OK;
}

// E^H without the coil sum: grid, the three inverse passes, and the z pass writes the
// cropped volume t[Nz][Ny][Nx][C] (scaled, not deapodised) into d_t2.
static mrg_status run_EH_crop_xyz(mrg_plan *p, const FrameTraj &ft, const float2 *y, cudaStream_t st) {
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Nx = g.N[0], Ny = g.N[1], Nz = g.N[2], Sz = g.S[2];
  MRG_TRY(run_EH_xy(p, ft, y, st));
  FftPass c;
  memset(&c, 0, sizeof(c));
  c.S = (int)Sz; c.sign = +1; c.mode = FFT_PLAIN;
  c.Lin = (int)Sz; c.in_off = 0; c.Lout = (int)Nz; c.out_off = g.og[2];
  c.inner = (int)(Nx * C); c.IB = plan_ib(p, 5, c.inner, C, false, c.S);
  c.nlines = Ny * Nx * C;
  c.in_ls = Ny * Nx * C; c.in_os = Nx * C; c.out_ls = Ny * Nx * C; c.out_os = Nx * C;
  c.scale = pass_scale(p, Sz);
  c.in = p->d_t1; c.out = p->d_t2; c.C = C;
  fft_vectorize(c);
  MRG_TRY(launch_fft(c, st));
  tmark(p, 4, st);
  tcollect(p, 4);
  return MRG_OK;
}

static mrg_status run_E_grid(mrg_plan *p, const float2 *X, const float2 *smap, cudaStream_t st) {
  if (p->C == 1) return run_E_grid_zxy(p, X, smap, st);
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Nx = g.N[0], Ny = g.N[1], Nz = g.N[2], Sx = g.S[0], Sy = g.S[1], Sz = g.S[2];
  const float *wx = p->d_win, *wy = p->d_win + Sx, *wz = p->d_win + Sx + Sy;
  // The passes run x, z, y so that set_image works on lines along x, where X and the
  // maps are contiguous: [Nz][Ny][Nx] -> t1 [Nz][Ny][Sx] -> t2 [Sz][Ny][Sx] -> grid [Sz][Sy][Sx].
  FftPass a;
  memset(&a, 0, sizeof(a));
  // x pass with set_image (src/gridFFT.cpp:972-986 + fft3 along x), input pruned to the crop
  a.S = (int)Sx; a.sign = -1; a.mode = FFT_SETIMG;
  a.Lin = (int)Nx; a.in_off = g.og[0]; a.Lout = (int)Sx; a.out_off = 0;
  a.inner = C; a.IB = plan_ib(p, 0, C, C, false, a.S); a.lfast = 0;
  a.nlines = Nz * Ny * C;
  a.in_ls = C; a.in_os = Nx * C; a.out_ls = C; a.out_os = Sx * C;
  a.scale = pass_scale(p, Sx);
  a.in = smap; a.smap = smap; a.has_smap = smap != nullptr; a.X = X; a.out = p->d_t1;
  a.wmode = 1; a.wdiv = Ny; a.wl = wx + g.og[0]; a.wo = wz + g.og[2]; a.wi = wy + g.og[1]; a.C = C;
  a.xp = p->fft_xp[0];
  tmark(p, 0, st);
  fft_vectorize(a);
  MRG_TRY(launch_fft(a, st));
  tmark(p, 1, st);
  // z pass: t1 [Nz][Ny][Sx] -> t2 [Sz][Ny][Sx], input pruned to the crop
  FftPass b;
  memset(&b, 0, sizeof(b));
  b.S = (int)Sz; b.sign = -1; b.mode = FFT_PLAIN;
  b.Lin = (int)Nz; b.in_off = g.og[2]; b.Lout = (int)Sz; b.out_off = 0;
  b.inner = (int)(Ny * Sx * C); b.IB = plan_ib(p, 1, b.inner, C, false, b.S);
  b.nlines = Ny * Sx * C;
  b.in_ls = Ny * Sx * C; b.in_os = 0; b.out_ls = Ny * Sx * C; b.out_os = 0;
  b.scale = pass_scale(p, Sz);
  b.in = p->d_t1; b.out = p->d_t2; b.C = C; b.xp = p->fft_xp[1]; b.err = p->d_err;
  fft_vectorize(b);
  MRG_TRY(launch_fft(b, st));
  tmark(p, 2, st);
  // y pass: t2 [Sz][Ny][Sx] -> grid [Sz][Sy][Sx]; the largest pass runs along y, whose rows
  // lie Sx*C apart (z rows are a whole plane apart)
  FftPass c;
  memset(&c, 0, sizeof(c));
  c.S = (int)Sy; c.sign = -1; c.mode = FFT_PLAIN;
  c.Lin = (int)Ny; c.in_off = g.og[1]; c.Lout = (int)Sy; c.out_off = 0;
  c.inner = (int)(Sx * C); c.IB = plan_ib(p, 2, c.inner, C, false, c.S);
  c.nlines = Sz * Sx * C;
  c.in_ls = Sx * C; c.in_os = Ny * Sx * C; c.out_ls = Sx * C; c.out_os = Sy * Sx * C;
  c.scale = pass_scale(p, Sy);
  c.in = p->d_t2; c.out = p->d_grid; c.C = C; c.xp = p->fft_xp[2]; c.err = p->d_err;
  fft_vectorize(c);
  MRG_TRY(launch_fft(c, st));
  return MRG_OK;
}

// E^H up to the z transform: grid, then the y and z inverse passes (cropping y and z);
// the result is t1 [Nz][Ny][Sx][C] in d_t1, so the last pass (x, cropped) can add into X
// and read the maps along contiguous lines.
static mrg_status run_EH_yz(mrg_plan *p, const FrameTraj &ft, const float2 *y, cudaStream_t st) {
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Ny = g.N[1], Nz = g.N[2], Sx = g.S[0], Sy = g.S[1], Sz = g.S[2];
  const GridConst gc = grid_const(p);
  tmark(p, 0, st);
  MRG_TRY(launch_grid(gc, ft, y, p->d_grid, st));  // src/gridFFT.cpp:1009-1164
  tmark(p, 1, st);
  // y pass: grid [Sz][Sy][Sx] -> t2 [Sz][Ny][Sx]
  FftPass a;
  memset(&a, 0, sizeof(a));
  a.S = (int)Sy; a.sign = +1; a.mode = FFT_PLAIN;
  a.Lin = (int)Sy; a.in_off = 0; a.Lout = (int)Ny; a.out_off = g.og[1];
  a.inner = (int)(Sx * C); a.IB = plan_ib(p, 3, a.inner, C, false, a.S);
  a.nlines = Sz * Sx * C;
  a.in_ls = Sx * C; a.in_os = Sy * Sx * C; a.out_ls = Sx * C; a.out_os = Ny * Sx * C;
  a.scale = pass_scale(p, Sy);
  a.in = p->d_grid; a.out = p->d_t2; a.C = C; a.xp = p->fft_xp[3]; a.err = p->d_err;
  fft_vectorize(a);
  MRG_TRY(launch_fft(a, st));
  tmark(p, 2, st);
  // z pass: t2 [Sz][Ny][Sx] -> t1 [Nz][Ny][Sx]
  FftPass b;
  memset(&b, 0, sizeof(b));
  b.S = (int)Sz; b.sign = +1; b.mode = FFT_PLAIN;
  b.Lin = (int)Sz; b.in_off = 0; b.Lout = (int)Nz; b.out_off = g.og[2];
  b.inner = (int)(Ny * Sx * C); b.IB = plan_ib(p, 4, b.inner, C, false, b.S);
  b.nlines = Ny * Sx * C;
  b.in_ls = Ny * Sx * C; b.in_os = 0; b.out_ls = Ny * Sx * C; b.out_os = 0;
  b.scale = pass_scale(p, Sz);
  b.in = p->d_t2; b.out = p->d_t1; b.C = C; b.xp = p->fft_xp[4]; b.err = p->d_err;
  fft_vectorize(b);
  MRG_TRY(launch_fft(b, st));
  tmark(p, 3, st);
  return MRG_OK;
}

static mrg_status run_EH(mrg_plan *p, const FrameTraj &ft, const float2 *y, const float2 *smap, float2 *X,
                         cudaStream_t st) {
  if (p->C == 1) return run_EH_xyz(p, ft, y, smap, X, st);
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Nx = g.N[0], Ny = g.N[1], Nz = g.N[2], Sx = g.S[0], Sy = g.S[1];
  const float *wx = p->d_win, *wy = p->d_win + Sx, *wz = p->d_win + Sx + Sy;
  MRG_TRY(run_EH_yz(p, ft, y, st));
  // x pass with accumulate (src/gridFFT.cpp:926-941): X[z][y][x] += sum_c ..., rows of X
  // written along x
  FftPass c;
  memset(&c, 0, sizeof(c));
  c.S = (int)Sx; c.sign = +1; c.mode = FFT_ACCUM;
  c.Lin = (int)Sx; c.in_off = 0; c.Lout = (int)Nx; c.out_off = g.og[0];
  c.inner = C; c.IB = plan_ib(p, 5, C, C, true, c.S);
  c.nlines = Nz * Ny * C;
  c.in_ls = C; c.in_os = Sx * C; c.out_ls = C; c.out_os = Nx * C;
  c.scale = pass_scale(p, Sx);
  c.in = p->d_t1; c.smap = smap; c.has_smap = smap != nullptr; c.acc = X;
  c.acc_atomic = (c.IB % C) != 0; c.acc_l = 1; c.acc_o = Nx;
  c.wmode = 1; c.wdiv = Ny; c.wl = wx + g.og[0]; c.wo = wz + g.og[2]; c.wi = wy + g.og[1]; c.C = C;
  c.xp = p->fft_xp[5];
  fft_vectorize(c);
  MRG_TRY(launch_fft(c, st));
  tmark(p, 4, st);
  tcollect(p, 4);
  return MRG_OK;
}

// E^H without the coil sum: grid, the three inverse passes, and the x pass writes the
// cropped volume t[Nz][Ny][Nx][C] (scaled, not deapodised) into d_t2.
static mrg_status run_EH_crop(mrg_plan *p, const FrameTraj &ft, const float2 *y, cudaStream_t st) {
  if (p->C == 1) return run_EH_crop_xyz(p, ft, y, st);
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Nx = g.N[0], Ny = g.N[1], Nz = g.N[2], Sx = g.S[0];
  MRG_TRY(run_EH_yz(p, ft, y, st));
  FftPass c;
  memset(&c, 0, sizeof(c));
  c.S = (int)Sx; c.sign = +1; c.mode = FFT_PLAIN;
  c.Lin = (int)Sx; c.in_off = 0; c.Lout = (int)Nx; c.out_off = g.og[0];
  c.inner = C; c.IB = (C == 1) ? pass_ib(C, C, c.S) : plan_ib(p, 5, C, C, false, c.S); c.lfast = (C == 1);
  c.nlines = Nz * Ny * C;
  c.in_ls = C; c.in_os = Sx * C; c.out_ls = C; c.out_os = Nx * C;
  c.scale = pass_scale(p, Sx);
  c.in = p->d_t1; c.out = p->d_t2; c.C = C;
  fft_vectorize(c);
  MRG_TRY(launch_fft(c, st));
  tmark(p, 4, st);
  tcollect(p, 4);
  return MRG_OK;
}

static mrg_status check_frame(const mrg_plan *p, int frame) {
  if (!p) {
    set_error("null plan");
    return MRG_ERR_INVALID;
  }
  if (frame < 0 || frame >= p->T) {
    set_error("frame index out of range");
    return MRG_ERR_INVALID;
  }
  if (p->frames[frame].M == 0) {
    set_error("no trajectory set for this frame");
    return MRG_ERR_STATE;
  }
  return MRG_OK;
}

static const float2 *plan_smap(const mrg_plan *p) { return p->has_smaps ? p->d_smap : nullptr; }

extern "C" {
static mrg_status ensure_solver(mrg_plan *p, bool fista);
}

// Picks 16 or 32 lines per CTA for each FFT pass, and for the x passes of multi-coil
// plans the persistent set_image / accumulate kernels or the one-tile ones, by timing one
// E and one E^H of this frame with each choice, using the per-stage event timing.  16
// lines halve a CTA's shared memory so more CTAs overlap their load, transform and store
// phases.
static mrg_status tune_fft(mrg_plan *p, const FrameTraj &ft, cudaStream_t st) {
  if (p->C > 32 || ft.nvalid == 0) return MRG_OK;
  MRG_TRY(ensure_solver(p, false));
  const float2 *sm = plan_smap(p) ? plan_smap(p) : (p->C > 1 ? p->d_grid : nullptr);
  const int was_on = p->timing_on;
  const int idx[6] = {0, 1, 2, 5, 6, 7};  // FFT stages among the eight timed stages
  float best[6];
  int pick[6];
  for (int k = 0; k < 6; k++) {
    best[k] = 1e30f;
    pick[k] = 0;
  }
  int pick_xp[6] = {0, 0, 0, 0, 0, 0};
  for (int cand = 0; cand < 6; cand++) {
    const int ib = (cand & 1) ? 16 : 0, xp = cand >> 1;
    for (int k = 0; k < 6; k++) {
      p->fft_ib[k] = ib;
      p->fft_xp[k] = xp;
    }
    MRG_TRY(mrg_set_timing(p, 1));
    for (int rep = 0; rep < 2; rep++) {
      MRG_TRY(run_E(p, ft, p->d_R, sm, nullptr, p->d_y, true, st));
      MRG_TRY(run_EH(p, ft, p->d_y, sm, p->d_L, st));
    }
    float t[8];
    int calls = 0;
    MRG_TRY(mrg_last_timings(p, t, &calls));
    for (int k = 0; k < 6; k++)
      if (t[idx[k]] < best[k]) {
        best[k] = t[idx[k]];
        pick[k] = ib;
        pick_xp[k] = xp;
      }
  }
  for (int k = 0; k < 6; k++) {
    p->fft_ib[k] = pick[k];
    p->fft_xp[k] = pick_xp[k];
  }
  // then, with those shapes, the plain persistent passes' tiles copied by tensor maps
  for (int k = 0; k < 6; k++) p->fft_xp[k] = pick_xp[k] | 4;
  MRG_TRY(mrg_set_timing(p, 1));
  for (int rep = 0; rep < 2; rep++) {
    MRG_TRY(run_E(p, ft, p->d_R, sm, nullptr, p->d_y, true, st));
    MRG_TRY(run_EH(p, ft, p->d_y, sm, p->d_L, st));
  }
  {
    float t[8];
    int calls = 0;
    MRG_TRY(mrg_last_timings(p, t, &calls));
    for (int k = 0; k < 6; k++) p->fft_xp[k] = t[idx[k]] < best[k] ? (pick_xp[k] | 4) : pick_xp[k];
  }
  const mrg_status chk = plan_check(p, st);
  if (chk == MRG_ERR_TIMEOUT) {  // a tensor-map copy's wait ran out: keep the 16-byte copies
    for (int k = 0; k < 6; k++) p->fft_xp[k] = pick_xp[k];
  } else {
    MRG_TRY(chk);
  }
  p->fft_tuned = true;
  return mrg_set_timing(p, was_on);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void mrg_config_default(mrg_config *cfg) {
  if (!cfg) return;
  cfg->overgrid = 1.5f;
  cfg->dwin = -1.0f;
  cfg->kernel_type = MRG_KERNEL_KAISER;
  cfg->k_rad = 9999.0f;
  cfg->time_grid = 0;
  cfg->tile = 0;
  cfg->max_pairs = 0;
  cfg->kernel_eval = 0;
  cfg->grid_mode = 0;
  cfg->fft_norm = 0;
}

const char *mrg_last_error(void) { return g_err.c_str(); }

int64_t mrg_kernel_launches(void) { return g_launches.load(); }

mrg_status mrg_plan_create(const mrg_config *cfg_in, int Nx, int Ny, int Nz, int ncoil, int nframes, mrg_plan **out) {
  if (!out) {
    set_error("out is NULL");
    return MRG_ERR_INVALID;
  }
  *out = nullptr;
  if (ncoil <= 0 || nframes <= 0) {
    set_error("sizes must be positive");
    return MRG_ERR_INVALID;
  }
  mrg_config cfg;
  if (cfg_in) cfg = *cfg_in; else mrg_config_default(&cfg);
  if (!config_ok(cfg, Nx, Ny, Nz)) return MRG_ERR_INVALID;
  mrg_plan *p = new mrg_plan();
  p->cfg = cfg;
  p->C = ncoil;
  p->T = nframes;
  build_geometry(p->geo, cfg, Nx, Ny, Nz);
  for (int d = 0; d < 3; d++) {
    if (!fft_size_supported(p->geo.S[d])) {
      set_error("oversampled size " + std::to_string(p->geo.S[d]) + " not supported by this build");
      delete p;
      return MRG_ERR_UNSUPPORTED;
    }
    if (p->geo.dwin[d] > 2.5f) {
      set_error("kernel half width above 2.5 not supported by this build");
      delete p;
      return MRG_ERR_UNSUPPORTED;
    }
  }
  p->B = cfg.tile > 0 ? cfg.tile : 2;
  if (p->geo.S[0] % p->B || p->geo.S[1] % p->B || p->geo.S[2] % p->B || p->B < 2 || p->B > 16) {
    set_error("tile must be 2..16 and divide the grid");
    delete p;
    return MRG_ERR_INVALID;
  }
  p->max_pairs = cfg.max_pairs > 0 ? cfg.max_pairs : 4096;
  p->nimg = (int64_t)Nx * Ny * Nz;
  p->frames.resize(nframes);
  mrg_status rs = fft_init_device();
  const int64_t S3 = (int64_t)p->geo.S[0] * p->geo.S[1] * p->geo.S[2];
  // E runs x, z, y (and E^H y, z, x): t1 = [Nz][Ny][Sx][C], t2 = [Sz][Ny][Sx][C]; one coil
  // keeps the z, y, x order: t1 = [Sz][Ny][Nx], t2 = [Sz][Sy][Nx]
  const int64_t t2n = std::max((int64_t)p->geo.S[2] * Ny * p->geo.S[0], (int64_t)Nx * p->geo.S[1] * p->geo.S[2]);
  const int64_t t1n = std::max((int64_t)Nz * Ny * p->geo.S[0], (int64_t)Nx * Ny * p->geo.S[2]);
  auto fail = [&](mrg_status s) {
    mrg_plan_destroy(p);
    return s;
  };
  if (rs != MRG_OK) return fail(rs);
#define ALLOC(ptr, bytes)                                                             \
  do {                                                                                \
    if (cudaMalloc((void **)&(ptr), (bytes)) != cudaSuccess) {                        \
      cudaGetLastError();                                                             \
      set_error(std::string("device allocation failed: ") + #ptr);                   \
      return fail(MRG_ERR_NOMEM);                                                     \
    }                                                                                 \
  } while (0)
  ALLOC(p->d_lut, sizeof(float) * 3 * p->geo.lut_len);
  ALLOC(p->d_win, sizeof(float) * (p->geo.S[0] + p->geo.S[1] + p->geo.S[2]));
  ALLOC(p->d_grid, sizeof(float2) * S3 * ncoil);
  ALLOC(p->d_t2, sizeof(float2) * t2n * ncoil);
  ALLOC(p->d_t1, sizeof(float2) * t1n * ncoil);
  ALLOC(p->d_sc, sizeof(Scalars));
  ALLOC(p->d_err, sizeof(int));
  if (cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) {
    set_error("error word initialisation failed");
    return fail(MRG_ERR_CUDA);
  }
  p->nblk = reduce_blocks(p->nimg * nframes);
  ALLOC(p->d_part, sizeof(double) * 3 * p->nblk);
#undef ALLOC
  std::vector<float> lut(3 * (size_t)p->geo.lut_len), win;
  for (int d = 0; d < 3; d++) std::copy(p->geo.lut[d].begin(), p->geo.lut[d].end(), lut.begin() + (size_t)d * p->geo.lut_len);
  for (int d = 0; d < 3; d++) win.insert(win.end(), p->geo.win[d].begin(), p->geo.win[d].end());
  if (cudaMemcpy(p->d_lut, lut.data(), sizeof(float) * lut.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->d_win, win.data(), sizeof(float) * win.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("table upload failed");
    return fail(MRG_ERR_CUDA);
  }
  if (cfg.time_grid) {
    const mrg_status ts = mrg_set_timing(p, 1);
    if (ts != MRG_OK) return fail(ts);
  }
  *out = p;
  return MRG_OK;
}

mrg_status mrg_plan_destroy(mrg_plan *p) {
  if (!p) return MRG_OK;
  for (auto &f : p->frames) traj_free(f);
  cudaFree(p->d_lut); cudaFree(p->d_win); cudaFree(p->d_grid); cudaFree(p->d_t2); cudaFree(p->d_t1);
  cudaFree(p->d_smap); cudaFree(p->d_y); cudaFree(p->d_R); cudaFree(p->d_P); cudaFree(p->d_L); cudaFree(p->d_Xo);
  cudaFree(p->d_part); cudaFree(p->d_sc); cudaFree(p->d_resid); cudaFree(p->d_err);
  for (int k = 0; k < 4; k++) cudaFree(p->d_stage[k]);
  if (p->cg_exec) cudaGraphExecDestroy(p->cg_exec);
  for (int k = 0; k < 5; k++)
    if (p->tev[k]) cudaEventDestroy(p->tev[k]);
  thr_free(p->thr);
  llr_free(p->llr);
  cudaFree(p->d_wshift);
  cudaFree(p->d_lshift);
  cudaFree(p->d_thr);
  delete p;
  return MRG_OK;
}

mrg_status mrg_plan_info(const mrg_plan *p, int S[3], int og[3], float grid[3], float beta[3], float dwin[3],
                         int *lut_len) {
  if (!p) {
    set_error("null plan");
    return MRG_ERR_INVALID;
  }
  for (int d = 0; d < 3; d++) {
    if (S) S[d] = p->geo.S[d];
    if (og) og[d] = p->geo.og[d];
    if (grid) grid[d] = p->geo.grid[d];
    if (beta) beta[d] = p->geo.beta[d];
    if (dwin) dwin[d] = p->geo.dwin[d];
  }
  if (lut_len) *lut_len = p->geo.lut_len;
  return MRG_OK;
}

mrg_status mrg_get_tables(const mrg_plan *p, float *lut, float *win) {
  if (!p) {
    set_error("null plan");
    return MRG_ERR_INVALID;
  }
  size_t o = 0;
  for (int d = 0; d < 3; d++) {
    if (lut) memcpy(lut + (size_t)d * p->geo.lut_len, p->geo.lut[d].data(), sizeof(float) * p->geo.lut_len);
    if (win) memcpy(win + o, p->geo.win[d].data(), sizeof(float) * p->geo.S[d]);
    o += p->geo.S[d];
  }
  return MRG_OK;
}

mrg_status mrg_set_smaps(mrg_plan *p, const void *smaps, int64_t coil_stride, void *stream) {
  if (!p || !smaps) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  if (coil_stride < p->nimg && p->C > 1) {
    set_error("coil_stride smaller than one image");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (!p->d_smap) MRG_CUDA(cudaMalloc(&p->d_smap, sizeof(float2) * p->nimg * p->C));
  void *src;
  bool staged;
  const size_t bytes = sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + p->nimg);
  MRG_TRY(dev_view(p, 0, smaps, bytes, true, st, &src, &staged));
  MRG_TRY(launch_interleave((const float2 *)src, coil_stride, p->C, p->nimg, p->d_smap, st));
  if (staged) MRG_CUDA(cudaStreamSynchronize(st));
  p->has_smaps = true;
  return MRG_OK;
}

mrg_status mrg_set_traj(mrg_plan *p, int frame, const float *kx, const float *ky, const float *kz, const float *kw,
                        int64_t M, void *stream) {
  if (!p || !kx || !ky || !kz || !kw) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  if (frame < 0 || frame >= p->T) {
    set_error("frame index out of range");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = sizeof(float) * (size_t)M;
  void *dx, *dy, *dz, *dw;
  bool s0, s1, s2, s3;
  MRG_TRY(dev_view(p, 0, kx, bytes, true, st, &dx, &s0));
  MRG_TRY(dev_view(p, 1, ky, bytes, true, st, &dy, &s1));
  MRG_TRY(dev_view(p, 2, kz, bytes, true, st, &dz, &s2));
  MRG_TRY(dev_view(p, 3, kw, bytes, true, st, &dw, &s3));
  const GridConst gc = grid_const(p);
  // region pair lists only where the tensor-memory gridding kernel may run
  const bool regions = umma_supported(p->C) && (p->cfg.grid_mode == 0 || p->cfg.grid_mode == 3);
  MRG_TRY(traj_setup(gc, p->frames[frame], (const float *)dx, (const float *)dy, (const float *)dz,
                     (const float *)dw, M, p->max_pairs, regions, st));
  invalidate_graphs(p);
  MRG_TRY(ensure_y(p, (int64_t)p->frames[frame].nvalid * p->C));
  FrameTraj &ft = p->frames[frame];
  const bool reuse = p->cfg.tile == 0 && p->tuned && ft.nvalid <= 2 * p->tuned_nvalid &&
                     2 * ft.nvalid >= p->tuned_nvalid;
  // the block pair lists only where a block-based gridding kernel may run: the autotuner
  // times them, and a reused choice may be one of them
  if (!regions || !reuse || p->tuned_cc > -100 || p->cfg.tile != 0)
    MRG_TRY(build_block_pairs(gc, ft, p->max_pairs, st));
  if (p->cfg.tile == 0) {
    const int64_t nv = ft.nvalid;
    if (reuse) {
      ft.ungrid_G = p->tuned_G;
      ft.ungrid_spb = p->tuned_spb;
      ft.ungrid_cpl = p->tuned_cpl;
      ft.ungrid_uy = p->tuned_uy;
      ft.grid_cc = p->tuned_cc;
      ft.tune_ungrid_ms = p->tuned_ms[0];
      ft.tune_grid_ms = p->tuned_ms[1];
    } else {
      MRG_TRY(autotune_frame(gc, ft, p->d_grid, p->d_y, st));
      if (!p->fft_tuned) MRG_TRY(tune_fft(p, ft, st));
      p->tuned_G = ft.ungrid_G;
      p->tuned_spb = ft.ungrid_spb;
      p->tuned_cpl = ft.ungrid_cpl;
      p->tuned_uy = ft.ungrid_uy;
      p->tuned_cc = ft.grid_cc;
      p->tuned = true;
      p->tuned_nvalid = nv;
      p->tuned_ms[0] = ft.tune_ungrid_ms;
      p->tuned_ms[1] = ft.tune_grid_ms;
    }
  }
  return MRG_OK;
}

mrg_status mrg_frame_info(const mrg_plan *p, int frame, int64_t *M, int64_t *nvalid, int64_t *npairs,
                          int64_t *nitems, int64_t *ntaps) {
  MRG_TRY(check_frame(p, frame));
  const FrameTraj &ft = p->frames[frame];
  if (M) *M = ft.M;
  if (nvalid) *nvalid = ft.nvalid;
  const PairSet &ps = ft.blocks.built ? ft.blocks : ft.regions;
  if (npairs) *npairs = ps.npairs;
  if (nitems) *nitems = ps.nitems;
  if (ntaps) MRG_TRY(count_taps(ft, ntaps));
  return MRG_OK;
}

mrg_status mrg_frame_tuning(const mrg_plan *p, int frame, int out[5], float ms[2]) {
  MRG_TRY(check_frame(p, frame));
  const FrameTraj &ft = p->frames[frame];
  if (out) {
    out[0] = ft.ungrid_G;
    out[1] = ft.ungrid_spb;
    out[2] = ft.grid_cc;
    out[3] = ft.ungrid_cpl;
    out[4] = ft.ungrid_uy;
  }
  if (ms) {
    ms[0] = ft.tune_ungrid_ms;
    ms[1] = ft.tune_grid_ms;
  }
  return MRG_OK;
}

mrg_status mrg_fft_tuning(const mrg_plan *p, int ib[6], int xp[6]) {
  if (!p) {
    set_error("null plan");
    return MRG_ERR_INVALID;
  }
  for (int k = 0; k < 6; k++) {
    if (ib) ib[k] = p->fft_ib[k];
    if (xp) xp[k] = p->fft_xp[k];
  }
  return MRG_OK;
}

mrg_status mrg_set_fft_tuning(mrg_plan *p, const int ib[6], const int xp[6]) {
  if (!p) {
    set_error("null plan");
    return MRG_ERR_INVALID;
  }
  for (int k = 0; k < 6; k++) {
    if (ib && (ib[k] < 0 || ib[k] > 32)) {
      set_error("lines per CTA out of range (0..32)");
      return MRG_ERR_INVALID;
    }
    if (xp && (xp[k] < 0 || xp[k] > 6 || (xp[k] & 3) == 3)) {
      set_error("xp must be 0, 1 or 2, optionally | 4");
      return MRG_ERR_INVALID;
    }
  }
  for (int k = 0; k < 6; k++) {
    if (ib) p->fft_ib[k] = ib[k];
    if (xp) p->fft_xp[k] = xp[k];
  }
  p->fft_tuned = true;
  invalidate_graphs(p);
  return MRG_OK;
}

mrg_status mrg_frame_set_tuning(mrg_plan *p, int frame, const int in[5]) {
  MRG_TRY(check_frame(p, frame));
  if (!in) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  FrameTraj &ft = p->frames[frame];
  const int G = in[0], spb = in[1], cc = in[2], cpl = in[3], uy = in[4];
  const bool g_ok = (G == 1 || G == 2 || G == 4 || G == 8 || G == 16 || G == 32) ||
                    ((G == -1 || G == -2 || G == -4 || G == -8) && p->C % (-4 * G) == 0);
  if (!g_ok || spb < 1 || !(cpl == 1 || cpl == 2 || cpl == 4) || uy < 1 || uy > 3) {
    set_error("ungridding launch shape out of range");
    return MRG_ERR_INVALID;
  }
  if (!grid_cc_allowed(p->C, ft, cc)) {
    set_error("gridding launch shape not available for this plan's coil count and grid_mode");
    return MRG_ERR_INVALID;
  }
  if (cc > -100) MRG_TRY(build_block_pairs(grid_const(p), ft, p->max_pairs, (cudaStream_t)0));
  ft.ungrid_G = G;
  ft.ungrid_spb = spb;
  ft.grid_cc = cc;
  ft.ungrid_cpl = cpl;
  ft.ungrid_uy = uy;
  invalidate_graphs(p);
  return MRG_OK;
}

mrg_status mrg_set_data(mrg_plan *p, int frame, const void *data, int64_t coil_stride, void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (!data) {
    set_error("null data");
    return MRG_ERR_INVALID;
  }
  FrameTraj &ft = p->frames[frame];
  if (p->C > 1 && coil_stride < ft.M) {
    set_error("coil_stride smaller than the sample count");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  MRG_TRY(grow(ft.dsorted, ft.cap_dsorted, (int64_t)ft.nvalid * p->C));
  void *src;
  bool staged;
  const size_t bytes = sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + ft.M);
  MRG_TRY(dev_view(p, 0, data, bytes, true, st, &src, &staged));
  MRG_TRY(launch_gather_samples(ft, p->C, (const float2 *)src, coil_stride, ft.dsorted, st));
  if (staged) MRG_CUDA(cudaStreamSynchronize(st));
  ft.has_data = true;
  return MRG_OK;
}

mrg_status mrg_adjoint(mrg_plan *p, int frame, const void *data, int64_t coil_stride, void *X, void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (!data || !X) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  if (p->C > 1 && !p->has_smaps) {
    set_error("coil maps not set");
    return MRG_ERR_STATE;
  }
  const FrameTraj &ft = p->frames[frame];
  if (p->C > 1 && coil_stride < ft.M) {
    set_error("coil_stride smaller than the sample count");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  void *dd, *dX;
  bool sd, sX;
  MRG_TRY(dev_view(p, 0, data, sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + ft.M), true, st, &dd, &sd));
  MRG_TRY(dev_view(p, 1, X, sizeof(float2) * p->nimg, true, st, &dX, &sX));
  MRG_TRY(launch_gather_samples(ft, p->C, (const float2 *)dd, coil_stride, p->d_y, st, true));
  MRG_TRY(run_EH(p, ft, p->d_y, plan_smap(p), (float2 *)dX, st));
  if (sX) {
    MRG_CUDA(cudaMemcpyAsync(X, dX, sizeof(float2) * p->nimg, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sX ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_forward(mrg_plan *p, int frame, const void *X, void *data, int64_t coil_stride, const void *diff,
                       void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (!data || !X) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  if (p->C > 1 && !p->has_smaps) {
    set_error("coil maps not set");
    return MRG_ERR_STATE;
  }
  const FrameTraj &ft = p->frames[frame];
  if (p->C > 1 && coil_stride < ft.M) {
    set_error("coil_stride smaller than the sample count");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t dbytes = sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + ft.M);
  void *dX, *dd, *ddf = nullptr;
  bool sX, sd, sdf = false;
  MRG_TRY(dev_view(p, 0, X, sizeof(float2) * p->nimg, true, st, &dX, &sX));
  MRG_TRY(dev_view(p, 1, data, dbytes, false, st, &dd, &sd));
  float2 *dsort = nullptr;
  if (diff) {
    // the sorted copy of diff lives behind the samples in the y buffer
    MRG_TRY(dev_view(p, 2, diff, dbytes, true, st, &ddf, &sdf));
    const int64_t ny = std::max<int64_t>(1, (int64_t)ft.nvalid * p->C);
    MRG_TRY(ensure_y(p, 2 * ny));
    dsort = p->d_y + ny;
    MRG_TRY(launch_gather_samples(ft, p->C, (const float2 *)ddf, coil_stride, dsort, st));
  }
  MRG_TRY(run_E(p, ft, (const float2 *)dX, plan_smap(p), dsort, p->d_y, false, st));
  MRG_TRY(launch_scatter_samples(ft, p->C, p->d_y, (float2 *)dd, coil_stride, st));
  if (sd) {
    MRG_CUDA(cudaMemcpyAsync(data, dd, dbytes, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sd ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_normal(mrg_plan *p, int frame, const void *X, void *out, void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (!X || !out) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  if (p->C > 1 && !p->has_smaps) {
    set_error("coil maps not set");
    return MRG_ERR_STATE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  void *dX, *dO;
  bool sX, sO;
  MRG_TRY(dev_view(p, 0, X, sizeof(float2) * p->nimg, true, st, &dX, &sX));
  MRG_TRY(dev_view(p, 1, out, sizeof(float2) * p->nimg, false, st, &dO, &sO));
  const FrameTraj &ft = p->frames[frame];
  MRG_TRY(launch_zero(dO, sizeof(float2) * p->nimg, st));
  MRG_TRY(run_E(p, ft, (const float2 *)dX, plan_smap(p), nullptr, p->d_y, true, st));
  MRG_TRY(run_EH(p, ft, p->d_y, plan_smap(p), (float2 *)dO, st));
  if (sO) {
    MRG_CUDA(cudaMemcpyAsync(out, dO, sizeof(float2) * p->nimg, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sO ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_adjoint_coil(mrg_plan *p, int frame, const void *smap, const void *data, void *X, void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (p->C != 1) {
    set_error("per-coil calls need a single-coil plan");
    return MRG_ERR_INVALID;
  }
  if (!data || !X) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const FrameTraj &ft = p->frames[frame];
  void *dd, *dX, *ds;
  bool sd, sX, ss;
  MRG_TRY(dev_view(p, 0, data, sizeof(float2) * (size_t)ft.M, true, st, &dd, &sd));
  MRG_TRY(dev_view(p, 1, X, sizeof(float2) * p->nimg, true, st, &dX, &sX));
  MRG_TRY(dev_view(p, 2, smap, sizeof(float2) * p->nimg, true, st, &ds, &ss));
  MRG_TRY(launch_gather_samples(ft, 1, (const float2 *)dd, 0, p->d_y, st, true));
  MRG_TRY(run_EH(p, ft, p->d_y, (const float2 *)ds, (float2 *)dX, st));
  if (sX) {
    MRG_CUDA(cudaMemcpyAsync(X, dX, sizeof(float2) * p->nimg, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sX ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_forward_coil(mrg_plan *p, int frame, const void *X, const void *smap, void *data, const void *diff,
                            void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (p->C != 1) {
    set_error("per-coil calls need a single-coil plan");
    return MRG_ERR_INVALID;
  }
  if (!data || !X) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const FrameTraj &ft = p->frames[frame];
  const size_t dbytes = sizeof(float2) * (size_t)ft.M;
  void *dX, *ds, *dd;
  bool sX, ss, sd;
  MRG_TRY(dev_view(p, 0, X, sizeof(float2) * p->nimg, true, st, &dX, &sX));
  MRG_TRY(dev_view(p, 1, smap, sizeof(float2) * p->nimg, true, st, &ds, &ss));
  MRG_TRY(dev_view(p, 2, data, dbytes, false, st, &dd, &sd));
  float2 *dsort = nullptr;
  if (diff) {
    void *ddf;
    bool sdf;
    MRG_TRY(dev_view(p, 3, diff, dbytes, true, st, &ddf, &sdf));
    const int64_t ny = std::max<int64_t>(1, (int64_t)ft.nvalid);
    MRG_TRY(ensure_y(p, 2 * ny));
    dsort = p->d_y + ny;
    MRG_TRY(launch_gather_samples(ft, 1, (const float2 *)ddf, 0, dsort, st));
  }
  MRG_TRY(run_E(p, ft, (const float2 *)dX, (const float2 *)ds, dsort, p->d_y, false, st));
  MRG_TRY(launch_scatter_samples(ft, 1, p->d_y, (float2 *)dd, 0, st));
  if (sd) {
    MRG_CUDA(cudaMemcpyAsync(data, dd, dbytes, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sd ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_set_k_rad(mrg_plan *p, float k_rad, void *stream) {
  if (!p || !(k_rad > 0.0f)) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  p->geo.k_rad = k_rad;
  p->cfg.k_rad = k_rad;
  const GridConst gc = grid_const(p);
  for (auto &ft : p->frames) MRG_TRY(launch_retaper(gc, ft, st));
  return MRG_OK;
}

// Shared front of the map-free adjoints: weighted gather of every coil's samples and
// E^H up to the cropped, transformed volume in d_t2.
static mrg_status adjoint_crop(mrg_plan *p, int frame, const void *data, int64_t coil_stride, cudaStream_t st) {
  MRG_TRY(check_frame(p, frame));
  if (!data) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  const FrameTraj &ft = p->frames[frame];
  if (p->C > 1 && coil_stride < ft.M) {
    set_error("coil_stride smaller than the sample count");
    return MRG_ERR_INVALID;
  }
  void *dd;
  bool sd;
  MRG_TRY(dev_view(p, 0, data, sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + ft.M), true, st, &dd, &sd));
  MRG_TRY(launch_gather_samples(ft, p->C, (const float2 *)dd, coil_stride, p->d_y, st, true));
  return run_EH_crop(p, ft, p->d_y, st);
}

mrg_status mrg_adjoint_coils(mrg_plan *p, int frame, const void *data, int64_t coil_stride, void *images,
                             int64_t image_stride, void *stream) {
  if (!p || !images) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  if (p->C > 1 && image_stride < p->nimg) {
    set_error("image_stride smaller than one image");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t vs = p->C > 1 ? image_stride : p->nimg;
  const size_t ibytes = sizeof(float2) * (size_t)(vs * (p->C - 1) + p->nimg);
  MRG_TRY(adjoint_crop(p, frame, data, coil_stride, st));
  void *dI;
  bool sI;
  MRG_TRY(dev_view(p, 1, images, ibytes, true, st, &dI, &sI));
  const Geometry &g = p->geo;
  const float *wx = p->d_win + g.og[0], *wy = p->d_win + g.S[0] + g.og[1], *wz = p->d_win + g.S[0] + g.S[1] + g.og[2];
  MRG_TRY(launch_coil_images(p->d_t2, p->C, g.N, wx, wy, wz, (float2 *)dI, 1, vs, true, st));
  if (sI) {
    MRG_CUDA(cudaMemcpyAsync(images, dI, ibytes, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sI ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_adjoint_sos(mrg_plan *p, int frame, const void *data, int64_t coil_stride, void *X, void *stream) {
  if (!p || !X) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  MRG_TRY(adjoint_crop(p, frame, data, coil_stride, st));
  void *dX;
  bool sX;
  MRG_TRY(dev_view(p, 1, X, sizeof(float2) * p->nimg, true, st, &dX, &sX));
  const Geometry &g = p->geo;
  const float *wx = p->d_win + g.og[0], *wy = p->d_win + g.S[0] + g.og[1], *wz = p->d_win + g.S[0] + g.S[1] + g.og[2];
  MRG_TRY(launch_sos_images(p->d_t2, p->C, g.N, wx, wy, wz, (float2 *)dX, st));
  if (sX) {
    MRG_CUDA(cudaMemcpyAsync(X, dX, sizeof(float2) * p->nimg, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sX ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_lowres_smaps(mrg_plan *p, int frame, const void *data, int64_t coil_stride, float smap_res,
                            const float blur[3], void *smaps_out, int64_t out_stride, void *stream) {
  if (!p || !(smap_res > 0.0f)) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  if (smaps_out && p->C > 1 && out_stride < p->nimg) {
    set_error("out_stride smaller than one image");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (!p->d_smap) MRG_CUDA(cudaMalloc(&p->d_smap, sizeof(float2) * p->nimg * p->C));
  const float k_rad = p->geo.k_rad;
  MRG_TRY(mrg_set_k_rad(p, smap_res, stream));  // gridding.k_rad = smap_res (src/recon_lib.cpp:2738)
  const mrg_status rs = adjoint_crop(p, frame, data, coil_stride, st);
  MRG_TRY(mrg_set_k_rad(p, k_rad, stream));  // restored afterwards (src/recon_lib.cpp:2786)
  MRG_TRY(rs);
  const Geometry &g = p->geo;
  const float *wx = p->d_win + g.og[0], *wy = p->d_win + g.S[0] + g.og[1], *wz = p->d_win + g.S[0] + g.S[1] + g.og[2];
  // coil images straight into the plan's interleaved maps [v][C]
  MRG_TRY(launch_coil_images(p->d_t2, p->C, g.N, wx, wy, wz, p->d_smap, p->C, 1, false, st));
  const float nob[3] = {0.f, 0.f, 0.f};
  MRG_TRY(gaussian_blur_ex(p->d_smap, p->C, g.N, p->C, 1, blur ? blur : nob, st));
  MRG_TRY(sos_normalize_ex(p->d_smap, p->C, p->nimg, p->C, 1, st));
  if (!p->has_smaps) invalidate_graphs(p);
  p->has_smaps = true;
  if (smaps_out) {
    const int64_t vs = p->C > 1 ? out_stride : p->nimg;
    const size_t obytes = sizeof(float2) * (size_t)(vs * (p->C - 1) + p->nimg);
    void *dO;
    bool sO;
    MRG_TRY(dev_view(p, 1, smaps_out, obytes, false, st, &dO, &sO));
    MRG_TRY(launch_deinterleave(p->d_smap, p->C, p->nimg, (float2 *)dO, vs, st));
    if (sO) {
      MRG_CUDA(cudaMemcpyAsync(smaps_out, dO, obytes, cudaMemcpyDeviceToHost, st));
      MRG_CUDA(cudaStreamSynchronize(st));
    }
  }
  return MRG_OK;
}

mrg_status mrg_fft3(mrg_plan *p, void *grid, int sign, void *stream) {
  if (!p || !grid || (sign != -1 && sign != 1)) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const Geometry &g = p->geo;
  const int C = p->C;
  const int64_t Sx = g.S[0], Sy = g.S[1], Sz = g.S[2];
  const size_t bytes = sizeof(float2) * (size_t)Sx * Sy * Sz * C;
  void *dG;
  bool sG;
  MRG_TRY(dev_view(p, 0, grid, bytes, true, st, &dG, &sG));
  float2 *G = (float2 *)dG;
  // axis d: lines of S[d] points, element stride ls, `inner` lines per outer row of stride os
  auto pass = [&](int d) -> mrg_status {
    const int64_t S = g.S[d];
    const int64_t ls = d == 0 ? C : (d == 1 ? Sx * C : Sy * Sx * C);
    const int64_t inner = ls, outer = (Sx * Sy * Sz * C) / (S * ls);
    FftPass a;
    memset(&a, 0, sizeof(a));
    a.S = (int)S; a.sign = sign; a.mode = FFT_PLAIN;
    a.Lin = (int)S; a.in_off = 0; a.Lout = (int)S; a.out_off = 0;
    a.inner = inner; a.IB = pass_ib(inner, C, a.S); a.lfast = 0;
    a.nlines = outer * inner;
    a.in_ls = ls; a.in_os = S * ls; a.out_ls = ls; a.out_os = S * ls;
    a.scale = pass_scale(p, S);
    a.in = G; a.out = G; a.C = C;
    fft_vectorize(a);
    return launch_fft(a, st);
  };
  const int order[3] = {2, 1, 0};  // do_fft: z, y, x; do_ifft: x, y, z
  for (int k = 0; k < 3; k++) MRG_TRY(pass(sign < 0 ? order[k] : order[2 - k]));
  if (sG) MRG_CUDA(cudaMemcpyAsync(grid, dG, bytes, cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

mrg_status mrg_grid(mrg_plan *p, int frame, const void *data, int64_t coil_stride, void *grid, void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (!data || !grid) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  const FrameTraj &ft = p->frames[frame];
  if (p->C > 1 && coil_stride < ft.M) {
    set_error("coil_stride smaller than the sample count");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const Geometry &g = p->geo;
  const size_t gbytes = sizeof(float2) * (size_t)g.S[0] * g.S[1] * g.S[2] * p->C;
  void *dd, *dG;
  bool sd, sG;
  MRG_TRY(dev_view(p, 0, data, sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + ft.M), true, st, &dd, &sd));
  MRG_TRY(dev_view(p, 1, grid, gbytes, false, st, &dG, &sG));
  // data * kw * taper in the sorted order, then the scatter (every grid point is written)
  MRG_TRY(launch_gather_samples(ft, p->C, (const float2 *)dd, coil_stride, p->d_y, st, true));
  const GridConst gc = grid_const(p);
  MRG_TRY(launch_grid(gc, ft, p->d_y, (float2 *)dG, st));
  if (sG) {
    MRG_CUDA(cudaMemcpyAsync(grid, dG, gbytes, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sG ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_ungrid(mrg_plan *p, int frame, const void *grid, void *data, int64_t coil_stride, const void *diff,
                      void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (!data || !grid) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  const FrameTraj &ft = p->frames[frame];
  if (p->C > 1 && coil_stride < ft.M) {
    set_error("coil_stride smaller than the sample count");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const Geometry &g = p->geo;
  const size_t gbytes = sizeof(float2) * (size_t)g.S[0] * g.S[1] * g.S[2] * p->C;
  const size_t dbytes = sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + ft.M);
  void *dG, *dd, *ddf = nullptr;
  bool sG, sd, sdf = false;
  MRG_TRY(dev_view(p, 0, grid, gbytes, true, st, &dG, &sG));
  MRG_TRY(dev_view(p, 1, data, dbytes, false, st, &dd, &sd));
  float2 *dsort = nullptr;
  if (diff) {  // the sorted copy of diff lives behind the samples in the y buffer
    MRG_TRY(dev_view(p, 2, diff, dbytes, true, st, &ddf, &sdf));
    const int64_t ny = std::max<int64_t>(1, (int64_t)ft.nvalid * p->C);
    MRG_TRY(ensure_y(p, 2 * ny));
    dsort = p->d_y + ny;
    MRG_TRY(launch_gather_samples(ft, p->C, (const float2 *)ddf, coil_stride, dsort, st));
  }
  const GridConst gc = grid_const(p);
  MRG_TRY(launch_ungrid(gc, ft, (const float2 *)dG, dsort, p->d_y, false, st));
  MRG_TRY(launch_scatter_samples(ft, p->C, p->d_y, (float2 *)dd, coil_stride, st));
  if (sd) {
    MRG_CUDA(cudaMemcpyAsync(data, dd, dbytes, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
  }
  return sd ? plan_check(p, st) : MRG_OK;
}

mrg_status mrg_espirit_smaps(mrg_plan *p, int frame, const void *data, int64_t coil_stride,
                             const mrg_espirit_params *params, const float blur[3], void *smaps_out,
                             int64_t out_stride, int *kept, void *stream) {
  if (!p || !params) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  if (smaps_out && p->C > 1 && out_stride < p->nimg) {
    set_error("out_stride smaller than one image");
    return MRG_ERR_INVALID;
  }
  for (int d = 0; d < 3; d++)
    if (!(params->kernel_radius[d] >= 0.0f) || params->kernel_radius[d] > 7.0f) {
      set_error("ESPIRiT kernel radius must be in [0, 7]");
      return MRG_ERR_INVALID;
    }
  cudaStream_t st = (cudaStream_t)stream;
  if (!p->d_smap) MRG_CUDA(cudaMalloc(&p->d_smap, sizeof(float2) * p->nimg * p->C));
  const Geometry &g = p->geo;
  if (p->C == 1) {  // one coil: the map is 1 (src/recon_lib.cpp:2703-2708)
    MRG_TRY(launch_fill(p->d_smap, p->nimg, make_float2(1.0f, 0.0f), st));
    if (kept) *kept = 0;
  } else {
    // coil images (gridding.forward per coil, k_rad unchanged: src/recon_lib.cpp:2737-2739)
    MRG_TRY(adjoint_crop(p, frame, data, coil_stride, st));
    const float *wx = p->d_win + g.og[0], *wy = p->d_win + g.S[0] + g.og[1], *wz = p->d_win + g.S[0] + g.S[1] + g.og[2];
    float2 *img = nullptr;
    MRG_CUDA(cudaMalloc(&img, sizeof(float2) * p->nimg * p->C));
    mrg_status s = launch_coil_images(p->d_t2, p->C, g.N, wx, wy, wz, img, p->C, 1, false, st);
    const float nob[3] = {0.f, 0.f, 0.f};
    if (s == MRG_OK) s = gaussian_blur_ex(img, p->C, g.N, p->C, 1, blur ? blur : nob, st);
    EspiritParams q;
    for (int d = 0; d < 3; d++) {
      q.kr_f[d] = params->kernel_radius[d];
      q.cr[d] = params->calib_radius[d];
    }
    q.svd_thresh = params->svd_thresh;
    q.square = params->square;
    q.sv_out = nullptr;
    q.sv_cap = 0;
    if (s == MRG_OK) s = espirit_maps(img, p->C, g.N, q, p->d_smap, kept, st);
    cudaStreamSynchronize(st);
    cudaFree(img);
    MRG_TRY(s);
  }
  if (!p->has_smaps) invalidate_graphs(p);
  p->has_smaps = true;
  if (smaps_out) {
    const int64_t vs = p->C > 1 ? out_stride : p->nimg;
    const size_t obytes = sizeof(float2) * (size_t)(vs * (p->C - 1) + p->nimg);
    void *dO;
    bool sO;
    MRG_TRY(dev_view(p, 1, smaps_out, obytes, false, st, &dO, &sO));
    MRG_TRY(launch_deinterleave(p->d_smap, p->C, p->nimg, (float2 *)dO, vs, st));
    if (sO) {
      MRG_CUDA(cudaMemcpyAsync(smaps_out, dO, obytes, cudaMemcpyDeviceToHost, st));
      MRG_CUDA(cudaStreamSynchronize(st));
    }
  }
  return MRG_OK;
}

static mrg_status capture(mrg_plan *p, const std::function<mrg_status(cudaStream_t)> &body, cudaGraphExec_t *exec);

// ---------------------------------------------------------------------------
// Differentiable E: loss, d loss / d image, d loss / d trajectory
// ---------------------------------------------------------------------------
mrg_status mrg_grad(mrg_plan *p, int frame, const void *X, const void *y, int64_t coil_stride, double *loss,
                    void *grad_x, float *grad_k, void *stream) {
  MRG_TRY(check_frame(p, frame));
  if (!X || !y || !grad_x || !grad_k) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  if (p->C > 1 && !p->has_smaps) {
    set_error("coil maps not set");
    return MRG_ERR_STATE;
  }
  if (p->cfg.kernel_type != MRG_KERNEL_KAISER) {
    set_error("the trajectory gradient needs the Kaiser-Bessel kernel (its analytic derivative)");
    return MRG_ERR_UNSUPPORTED;
  }
  FrameTraj &ft = p->frames[frame];
  if (p->C > 1 && coil_stride < ft.M) {
    set_error("coil_stride smaller than the sample count");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const GridConst gc = grid_const(p);
  if (!ft.sdw_valid) MRG_TRY(launch_sample_dweights(gc, ft, st));
  const size_t ybytes = sizeof(float2) * (size_t)(coil_stride * (p->C - 1) + ft.M);
  void *dX, *dy, *dgx, *dgk;
  bool sX, sy, sgx, sgk;
  MRG_TRY(dev_view(p, 0, X, sizeof(float2) * p->nimg, true, st, &dX, &sX));
  MRG_TRY(dev_view(p, 1, y, ybytes, true, st, &dy, &sy));
  MRG_TRY(dev_view(p, 2, grad_x, sizeof(float2) * p->nimg, false, st, &dgx, &sgx));
  MRG_TRY(dev_view(p, 3, grad_k, sizeof(float) * 3 * (size_t)ft.M, false, st, &dgk, &sgk));
  // E passes up to the oversampled grid (the ungrid step is replaced by the gradient gather)
  MRG_TRY(launch_zero(&p->d_sc->e, sizeof(double), st));
  MRG_TRY(launch_gather_samples(ft, p->C, (const float2 *)dy, coil_stride, p->d_y, st, false));
  MRG_TRY(run_E_grid(p, (const float2 *)dX, plan_smap(p), st));
  MRG_TRY(launch_ungrid_grad(gc, ft, p->d_grid, p->d_y, (const float2 *)dy, coil_stride, (float *)dgk,
                             &p->d_sc->e, st));
  // grad_x = E^*(2r): the adjoint without density weights or taper
  MRG_TRY(launch_zero(dgx, sizeof(float2) * p->nimg, st));
  MRG_TRY(run_EH(p, ft, p->d_y, plan_smap(p), (float2 *)dgx, st));
  if (loss) MRG_CUDA(cudaMemcpyAsync(loss, &p->d_sc->e, sizeof(double), cudaMemcpyDeviceToHost, st));
  if (sgx) MRG_CUDA(cudaMemcpyAsync(grad_x, dgx, sizeof(float2) * p->nimg, cudaMemcpyDeviceToHost, st));
  if (sgk) MRG_CUDA(cudaMemcpyAsync(grad_k, dgk, sizeof(float) * 3 * (size_t)ft.M, cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return plan_check(p, st);
}

// ---------------------------------------------------------------------------
// SENSE-CG (src/recon_lib.cpp:1523-1759)
// ---------------------------------------------------------------------------
static mrg_status ensure_solver(mrg_plan *p, bool fista) {
  const size_t vb = sizeof(float2) * (size_t)p->nimg * p->T;
  if (!p->d_R) MRG_CUDA(cudaMalloc(&p->d_R, vb));
  if (!p->d_P) MRG_CUDA(cudaMalloc(&p->d_P, vb));
  if (!p->d_L) MRG_CUDA(cudaMalloc(&p->d_L, vb));
  if (fista && !p->d_Xo) MRG_CUDA(cudaMalloc(&p->d_Xo, vb));
  return MRG_OK;
}

static mrg_status ensure_resid(mrg_plan *p, int n) {
  if (p->resid_cap >= n) return MRG_OK;
  invalidate_graphs(p);
  cudaFree(p->d_resid);
  p->d_resid = nullptr;
  MRG_CUDA(cudaMalloc(&p->d_resid, sizeof(double) * std::max(n, 1)));
  p->resid_cap = n;
  return MRG_OK;
}

// LHS = sum_c E^H W E P per frame, then the vector updates of one CG iteration.
static mrg_status cg_iteration(mrg_plan *p, float2 *X, cudaStream_t st) {
  const int64_t n = p->nimg;
  const int64_t nt = n * p->T;
  for (int t = 0; t < p->T; t++) {
    const FrameTraj &ft = p->frames[t];
    float2 *Lt = p->d_L + t * n;
    MRG_TRY(launch_zero(Lt, sizeof(float2) * n, st));
    MRG_TRY(run_E(p, ft, p->d_P + t * n, plan_smap(p), nullptr, p->d_y, true, st));
    MRG_TRY(run_EH(p, ft, p->d_y, plan_smap(p), Lt, st));
  }
  MRG_TRY(cg_dots(p->d_R, p->d_P, p->d_L, nt, p->d_part, p->nblk, p->d_sc, st));
  MRG_TRY(cg_update(X, p->d_R, p->d_P, p->d_L, nt, p->d_part, p->nblk, p->d_sc, p->d_resid, st));
  MRG_TRY(cg_pupdate(p->d_P, p->d_R, nt, p->d_sc, st));
  return MRG_OK;
}

static mrg_status cg_ready(mrg_plan *p) {
  for (int t = 0; t < p->T; t++) {
    MRG_TRY(check_frame(p, t));
    if (!p->frames[t].has_data) {
      set_error("k-space data not set for a frame");
      return MRG_ERR_STATE;
    }
  }
  if (p->C > 1 && !p->has_smaps) {
    set_error("coil maps not set");
    return MRG_ERR_STATE;
  }
  return MRG_OK;
}

mrg_status mrg_cg_init(mrg_plan *p, int max_iter, void *X, void *stream) {
  if (!p || !X || max_iter < 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  if (!is_device_ptr(X)) {
    set_error("mrg_cg_init needs X in device memory (mrg_cg stages host buffers)");
    return MRG_ERR_INVALID;
  }
  MRG_TRY(cg_ready(p));
  cudaStream_t st = (cudaStream_t)stream;
  MRG_TRY(ensure_solver(p, false));
  MRG_TRY(ensure_resid(p, std::max(max_iter, 1)));
  const int64_t n = p->nimg, nt = n * p->T;
  float2 *Xd = (float2 *)X;
  // R = sum_c E^H W d, P = R, X = 0  (src/recon_lib.cpp:1537-1573)
  MRG_TRY(launch_zero(Xd, sizeof(float2) * nt, st));
  MRG_TRY(launch_zero(p->d_R, sizeof(float2) * nt, st));
  for (int t = 0; t < p->T; t++) {
    MRG_TRY(launch_weigh_samples(p->frames[t], p->C, p->frames[t].dsorted, p->d_y, st));
    MRG_TRY(run_EH(p, p->frames[t], p->d_y, plan_smap(p), p->d_R + t * n, st));
  }
  MRG_TRY(launch_copy(p->d_P, p->d_R, nt, st));
  Scalars z;
  memset(&z, 0, sizeof(z));
  MRG_CUDA(cudaMemcpyAsync(p->d_sc, &z, sizeof(Scalars), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return MRG_OK;
}

mrg_status mrg_cg_iterate(mrg_plan *p, int nit, void *X, int use_graph, void *stream) {
  if (!p || !X || nit < 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  if (!p->d_R) {
    set_error("mrg_cg_init not called");
    return MRG_ERR_STATE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  float2 *Xd = (float2 *)X;
  if (use_graph && !p->timing_on && nit > 0) {
    if (!p->cg_exec || p->cg_key[0] != X) {
      invalidate_graphs(p);
      const int64_t before = g_launches.load();
      MRG_TRY(capture(p, [&](cudaStream_t cs) { return cg_iteration(p, Xd, cs); }, &p->cg_exec));
      p->graph_kernels = g_launches.load() - before;  // captured, not launched
      g_launches.fetch_sub(p->graph_kernels);
      p->cg_key[0] = X;
    }
    for (int it = 0; it < nit; it++) {
      MRG_CUDA(cudaGraphLaunch(p->cg_exec, st));
      count_launch((int)p->graph_kernels);
    }
  } else {
    for (int it = 0; it < nit; it++) MRG_TRY(cg_iteration(p, Xd, st));
  }
  return MRG_OK;
}

mrg_status mrg_cg_residuals(mrg_plan *p, double *resid, int n, void *stream) {
  if (!p || (n > 0 && !resid) || n < 0 || n > p->resid_cap) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (n > 0) MRG_CUDA(cudaMemcpyAsync(resid, p->d_resid, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return plan_check(p, st);
}

mrg_status mrg_cg(mrg_plan *p, int max_iter, void *X, double *resid, int use_graph, void *stream) {
  if (!p || !X || max_iter < 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  MRG_TRY(cg_ready(p));
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nt = p->nimg * p->T;
  void *dX;
  bool sX;
  MRG_TRY(dev_view(p, 0, X, sizeof(float2) * nt, false, st, &dX, &sX));
  MRG_TRY(mrg_cg_init(p, max_iter, dX, stream));
  MRG_TRY(mrg_cg_iterate(p, max_iter, dX, use_graph, stream));
  p->last_iters = max_iter;
  if (resid && max_iter > 0) MRG_TRY(mrg_cg_residuals(p, resid, max_iter, stream));
  if (sX) MRG_CUDA(cudaMemcpyAsync(X, dX, sizeof(float2) * nt, cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return plan_check(p, st);
}

mrg_status mrg_set_timing(mrg_plan *p, int enable) {
  if (!p) {
    set_error("null plan");
    return MRG_ERR_INVALID;
  }
  if (enable && !p->tev[0])
    for (int k = 0; k < 5; k++) MRG_CUDA(cudaEventCreate(&p->tev[k]));
  p->timing_on = enable ? 1 : 0;
  memset(p->timings, 0, sizeof(p->timings));
  p->timing_calls = 0;
  return MRG_OK;
}

mrg_status mrg_last_timings(mrg_plan *p, float out[8], int *calls) {
  if (!p || !out) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  memcpy(out, p->timings, sizeof(p->timings));
  if (calls) *calls = p->timing_calls;
  memset(p->timings, 0, sizeof(p->timings));
  p->timing_calls = 0;
  return MRG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FISTA / IST (src/recon_lib.cpp:1761-2212)
// ---------------------------------------------------------------------------
struct FistaCtx {
  const mrg_fista_params *q;
  int N[3], L[3], max_level, bs[3];
  float2 *X;
};

static mrg_status capture(mrg_plan *p, const std::function<mrg_status(cudaStream_t)> &body, cudaGraphExec_t *exec) {
  cudaStream_t cs;
  MRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t graph;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaStreamDestroy(cs);
    set_error("stream capture failed to start");
    return MRG_ERR_CUDA;
  }
  const mrg_status cap = body(cs);
  const cudaError_t ee = cudaStreamEndCapture(cs, &graph);
  cudaStreamDestroy(cs);
  if (cap != MRG_OK) {
    if (ee == cudaSuccess) cudaGraphDestroy(graph);
    return cap;
  }
  if (ee != cudaSuccess) {
    set_error(std::string("stream capture failed: ") + cudaGetErrorString(ee));
    return MRG_ERR_CUDA;
  }
  const cudaError_t ie = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    *exec = nullptr;
    set_error(std::string("graph instantiate failed: ") + cudaGetErrorString(ie));
    return MRG_ERR_CUDA;
  }
  (void)p;
  return MRG_OK;
}

// One power-iteration step: X = E^H W E X / ||E^H W E X||, step = 1/||.||
// (src/recon_lib.cpp:1818-1906).
static mrg_status power_step(mrg_plan *p, float2 *X, cudaStream_t st) {
  const int64_t n = p->nimg, nt = n * p->T;
  MRG_TRY(launch_zero(p->d_R, sizeof(float2) * nt, st));
  for (int t = 0; t < p->T; t++) {
    MRG_TRY(run_E(p, p->frames[t], X + t * n, plan_smap(p), nullptr, p->d_y, true, st));
    MRG_TRY(run_EH(p, p->frames[t], p->d_y, plan_smap(p), p->d_R + t * n, st));
  }
  MRG_TRY(energy(p->d_R, nt, p->d_part, p->nblk, &p->d_sc->e, st));
  MRG_TRY(power_scale(X, p->d_R, nt, p->d_sc, st));
  return MRG_OK;
}

static mrg_status fista_iteration(mrg_plan *p, const FistaCtx &f, cudaStream_t st) {
  const mrg_fista_params &q = *f.q;
  const int64_t n = p->nimg, nt = n * p->T;
  float2 *X = f.X;
  MRG_TRY(fista_momentum(X, p->d_Xo, nt, p->d_sc, q.fista, st));  // fista_update
  MRG_TRY(launch_zero(p->d_R, sizeof(float2) * nt, st));
  for (int t = 0; t < p->T; t++) {  // R = E^H W (E x - d)
    MRG_TRY(run_E(p, p->frames[t], X + t * n, plan_smap(p), p->frames[t].dsorted, p->d_y, true, st));
    MRG_TRY(run_EH(p, p->frames[t], p->d_y, plan_smap(p), p->d_R + t * n, st));
  }
  MRG_TRY(grad_step(X, p->d_R, nt, p->d_sc, p->d_part, p->nblk, p->d_resid, st));  // X -= step R
  if (q.llr_alpha > 0.0f) {  // lranktime.update_threshold / thresh (src/recon_lib.cpp:2117-2121)
    MRG_TRY(llr_update_ex(X, p->T, f.N, f.bs, q.clear_amp, q.clear_t2, p->d_sc, 0, p->llr, st));
    MRG_TRY(llr_apply_ex(X, p->T, f.N, f.bs, q.llr_block_iter, q.llr_alpha, p->d_lshift, p->d_sc,
                         3 * q.llr_block_iter, 0, p->llr.smax, st));
  }
  if (q.use_threshold) {  // L1_threshold with cycle spinning (src/recon_lib.cpp:2491-2509)
    const float scale = (float)(1. / (float)q.cycle_spins);
    for (int spin = 0; spin < q.cycle_spins; spin++) {
      MRG_TRY(wavelet3d_ex(X, p->T, f.N, f.L, f.max_level, p->d_wshift, p->d_sc, 3 * q.cycle_spins, 3 * spin,
                           q.wave_type, 0, st));
      // a fixed threshold (use_threshold 2) was written to d_thr once, before the loop
      if (spin == 0 && q.use_threshold == 1) MRG_TRY(fraction_threshold(X, nt, q.thresh, scale, p->thr, p->d_thr, st));
      MRG_TRY(soft_threshold(X, nt, p->d_thr, st));
      MRG_TRY(wavelet3d_ex(X, p->T, f.N, f.L, f.max_level, p->d_wshift, p->d_sc, 3 * q.cycle_spins, 3 * spin,
                           q.wave_type, 1, st));
    }
  }
  MRG_TRY(bump_iteration(p->d_sc, st));
  return MRG_OK;
}

extern "C" mrg_status mrg_fista(mrg_plan *p, const mrg_fista_params *q, void *X, double *resid, float *step,
                                int use_graph, void *stream) {
  if (!p || !q || !X || q->max_iter < 0 || q->max_eig_iter < 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  // the per-iteration shift tables are sized max_iter x (cycle spins, block iterations) x 3
  if (q->max_iter > 100000 || q->max_eig_iter > 100000) {
    set_error("max_iter / max_eig_iter above 100000");
    return MRG_ERR_INVALID;
  }
  if (q->use_threshold && (q->cycle_spins < 1 || q->cycle_spins > 64 || q->wave_type < 0 || q->wave_type > 1)) {
    set_error("bad wavelet / cycle-spin parameters");
    return MRG_ERR_INVALID;
  }
  if (q->use_threshold < 0 || q->use_threshold > 2) {
    set_error("use_threshold must be 0 (none), 1 (fraction) or 2 (fixed)");
    return MRG_ERR_INVALID;
  }
  if (q->llr_alpha > 0.0f && (q->llr_block_iter < 1 || q->llr_block_iter > 64 || q->llr_block[0] < 1 ||
                              q->llr_block[1] < 1 || q->llr_block[2] < 1)) {
    set_error("bad low-rank block parameters");
    return MRG_ERR_INVALID;
  }
  const bool early_stop = q->early_stop_thresh > 0.0f;
  if (early_stop && q->early_stop_range < 1) {
    set_error("early_stop_range must be at least 1");
    return MRG_ERR_INVALID;
  }
  for (int t = 0; t < p->T; t++) {
    MRG_TRY(check_frame(p, t));
    if (!p->frames[t].has_data) {
      set_error("k-space data not set for a frame");
      return MRG_ERR_STATE;
    }
  }
  if (p->C > 1 && !p->has_smaps) {
    set_error("coil maps not set");
    return MRG_ERR_STATE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  MRG_TRY(ensure_solver(p, true));
  MRG_TRY(ensure_resid(p, std::max(q->max_iter, 1)));
  invalidate_graphs(p);
  const int64_t n = p->nimg, nt = n * p->T;
  FistaCtx f;
  f.q = q;
  for (int d = 0; d < 3; d++) {
    f.N[d] = p->geo.N[d];
    f.bs[d] = std::min(q->llr_block[d], f.N[d]);  // clear.cpp:246-248
  }
  wavelet_levels(f.N, q->wave_levels, f.L, &f.max_level);
  // rand() draws in the reference's order: per iteration the low-rank block
  // shifts (clear.cpp:408-415), then 3 wavelet shifts per cycle spin
  // (wavelet3D.cpp:443-448), after the max-eigen seeding draws.
  GlibcRand rng;
  rng.skip(q->rand_skip >= 0 ? q->rand_skip : 2 * nt);
  const int wN = q->wave_type == 0 ? 2 : 4;
  const int iters = std::max(q->max_iter, 1);
  std::vector<int> wsh((size_t)iters * 3 * std::max(q->cycle_spins, 1), 0);
  std::vector<int> lsh((size_t)iters * 3 * std::max(q->llr_block_iter, 1), 0);
  for (int it = 0; it < q->max_iter; it++) {
    if (q->llr_alpha > 0.0f)
      for (int b = 0; b < q->llr_block_iter; b++) {
        int *s3 = &lsh[((size_t)it * q->llr_block_iter + b) * 3];
        for (int d = 0; d < 3; d++) s3[d] = rng.next() % f.bs[d] - f.bs[d] / 2;
        if (q->llr_block_iter == 1) s3[0] = s3[1] = s3[2] = 0;
      }
    if (q->use_threshold)
      for (int sp = 0; sp < q->cycle_spins; sp++)
        for (int d = 0; d < 3; d++) wsh[((size_t)it * q->cycle_spins + sp) * 3 + d] = rng.next() % wN;
  }
  cudaFree(p->d_wshift);
  cudaFree(p->d_lshift);
  p->d_wshift = p->d_lshift = nullptr;
  MRG_CUDA(cudaMalloc(&p->d_wshift, sizeof(int) * wsh.size()));
  MRG_CUDA(cudaMalloc(&p->d_lshift, sizeof(int) * lsh.size()));
  MRG_CUDA(cudaMemcpyAsync(p->d_wshift, wsh.data(), sizeof(int) * wsh.size(), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaMemcpyAsync(p->d_lshift, lsh.data(), sizeof(int) * lsh.size(), cudaMemcpyHostToDevice, st));
  if (!p->d_thr) MRG_CUDA(cudaMalloc(&p->d_thr, sizeof(float)));
  if (q->use_threshold == 1) MRG_TRY(thr_alloc(p->thr, nt));
  if (q->use_threshold == 2) {
    // THRESHOLD::update_threshold, TH_FIXED: global_threshold = thresh * scale with the cycle-spin
    // scale 1/cycle_spins passed as float (src/threshold.cpp:196-198, src/recon_lib.cpp:2499-2501)
    const float scale = (float)(1.0 / (float)q->cycle_spins);
    const float fixed = (float)((double)q->thresh * (double)scale);
    MRG_CUDA(cudaMemcpy(p->d_thr, &fixed, sizeof(float), cudaMemcpyHostToDevice));
  }
  void *dX;
  bool sX;
  MRG_TRY(dev_view(p, 0, X, sizeof(float2) * nt, false, st, &dX, &sX));
  f.X = (float2 *)dX;
  Scalars z;
  memset(&z, 0, sizeof(z));
  z.step = 1.0f;
  MRG_CUDA(cudaMemcpyAsync(p->d_sc, &z, sizeof(Scalars), cudaMemcpyHostToDevice, st));
  // power iteration from the constant seed -0.5-0.5i (std::rand()/RAND_MAX is an
  // integer division, src/recon_lib.cpp:1809-1811)
  MRG_TRY(launch_fill(f.X, nt, make_float2(-0.5f, -0.5f), st));
  if (q->max_eig_iter > 0) {
    if (use_graph) {
      cudaGraphExec_t ge = nullptr;
      MRG_TRY(power_step(p, f.X, st));  // first step eagerly: sets kernel attributes outside capture
      MRG_CUDA(cudaStreamSynchronize(st));
      MRG_TRY(capture(p, [&](cudaStream_t cs) { return power_step(p, f.X, cs); }, &ge));
      mrg_status rs = MRG_OK;
      for (int it = 1; it < q->max_eig_iter && rs == MRG_OK; it++) {
        if (cudaGraphLaunch(ge, st) != cudaSuccess) rs = MRG_ERR_CUDA;
        count_launch();
      }
      cudaGraphExecDestroy(ge);
      if (rs != MRG_OK) {
        set_error("graph launch failed");
        return rs;
      }
    } else {
      for (int it = 0; it < q->max_eig_iter; it++) MRG_TRY(power_step(p, f.X, st));
    }
  }
  // X = 0, X_old = 0, iteration counter 0 (step kept)
  MRG_TRY(launch_zero(f.X, sizeof(float2) * nt, st));
  MRG_TRY(launch_zero(p->d_Xo, sizeof(float2) * nt, st));
  MRG_CUDA(cudaMemcpyAsync(&p->d_sc->it, &z.it, sizeof(int), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  // Early stop (src/recon_lib.cpp:2081-2087, :2154-2163): after each iteration the ratio of its
  // sum |R|^2 to iteration 0's joins the last early_stop_range ratios; the loop ends once
  // their standard deviation is below early_stop_thresh.  Checking reads one residual back
  // per iteration, so it runs only when a threshold is set.
  std::vector<float> diffs;
  double error0 = 0.0;
  auto stop_after = [&](int it) -> int {  // 1: stop, 0: go on, < 0: -(mrg_status)
    if (!early_stop) return 0;
    double r = 0.0;
    if (cudaMemcpyAsync(&r, p->d_resid + it, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      set_error("residual read-back failed");
      return -(int)MRG_ERR_CUDA;
    }
    if (it == 0) error0 = r;
    const float ratio = (float)(std::fabs(r) / error0);
    return early_stop_met(diffs, ratio, q->early_stop_range, q->early_stop_thresh) ? 1 : 0;
  };
  int done = 0;
  if (use_graph && q->max_iter > 1) {
    MRG_TRY(fista_iteration(p, f, st));  // iteration 0 eagerly, then replay the captured iteration
    MRG_CUDA(cudaStreamSynchronize(st));
    done = 1;
    int stop = stop_after(0);
    if (stop < 0) return (mrg_status)(-stop);
    if (!stop) {
      cudaGraphExec_t ge = nullptr;
      MRG_TRY(capture(p, [&](cudaStream_t cs) { return fista_iteration(p, f, cs); }, &ge));
      mrg_status rs = MRG_OK;
      for (int it = 1; it < q->max_iter && rs == MRG_OK; it++) {
        if (cudaGraphLaunch(ge, st) != cudaSuccess) {
          rs = MRG_ERR_CUDA;
          set_error("graph launch failed");
          break;
        }
        count_launch();
        done = it + 1;
        stop = stop_after(it);
        if (stop < 0) rs = (mrg_status)(-stop);
        if (stop) break;
      }
      cudaGraphExecDestroy(ge);
      if (rs != MRG_OK) return rs;
    }
  } else {
    for (int it = 0; it < q->max_iter; it++) {
      MRG_TRY(fista_iteration(p, f, st));
      done = it + 1;
      const int stop = stop_after(it);
      if (stop < 0) return (mrg_status)(-stop);
      if (stop) break;
    }
  }
  p->last_iters = done;
  if (resid && done > 0)
    MRG_CUDA(cudaMemcpyAsync(resid, p->d_resid, sizeof(double) * done, cudaMemcpyDeviceToHost, st));
  if (step) MRG_CUDA(cudaMemcpyAsync(step, &p->d_sc->step, sizeof(float), cudaMemcpyDeviceToHost, st));
  if (sX) MRG_CUDA(cudaMemcpyAsync(X, dX, sizeof(float2) * nt, cudaMemcpyDeviceToHost, st));
  MRG_CUDA(cudaStreamSynchronize(st));
  return plan_check(p, st);
}

// CLEAR (src/recon_lib.cpp:1025-1238).  The per-coil images XX, the gradients RR and
// E^H W E RR (one frame at a time) are [frame][voxel][coil] stacks, the layout the
// operators read coil maps in: E_c X_c is run as E of a unit image with "maps" X_c for
// all coils at once, and E_c^H of every coil comes out of the cropped adjoint transform.
extern "C" mrg_status mrg_clear(mrg_plan *p, const mrg_clear_params *q, void *X, void *coil_images, double *resid,
                                int *iters, void *stream) {
  if (!p || !q || !X || q->max_iter < 0 || q->block[0] < 1 || q->block[1] < 1 || q->block[2] < 1) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  if (q->max_iter > 100000) {  // the shift tables are sized per iteration
    set_error("max_iter above 100000");
    return MRG_ERR_INVALID;
  }
  if (q->alpha_coil != 0.0f && (q->block_iter < 1 || q->block_iter > 64 || q->rand_skip < 0)) {
    set_error("bad low-rank block parameters");
    return MRG_ERR_INVALID;
  }
  if (q->use_threshold &&
      (q->cycle_spins < 1 || q->cycle_spins > 64 || q->wave_type < 0 || q->wave_type > 1 || q->rand_skip < 0)) {
    set_error("bad wavelet / cycle-spin parameters");
    return MRG_ERR_INVALID;
  }
  if (p->C > 32) {
    set_error("CLEAR supports at most 32 coils");
    return MRG_ERR_UNSUPPORTED;
  }
  for (int t = 0; t < p->T; t++) {
    MRG_TRY(check_frame(p, t));
    if (!p->frames[t].has_data) {
      set_error("k-space data not set for a frame");
      return MRG_ERR_STATE;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  const Geometry &g = p->geo;
  const int C = p->C, T = p->T;
  const int64_t n = p->nimg, nc = n * C, ntc = nc * T;
  int bs[3];
  for (int d = 0; d < 3; d++) bs[d] = std::min(q->block[d], g.N[d]);  // clear.cpp:109-112
  const int64_t nb64 = coil_llr_blocks(g.N, bs);
  if (nb64 > (int64_t)(1 << 30)) {
    set_error("too many coil low-rank blocks (" + std::to_string(nb64) + ")");
    return MRG_ERR_UNSUPPORTED;
  }
  const int nb = (int)nb64;
  int np2 = 1;
  while (np2 < nb) np2 <<= 1;
  const int nblk = reduce_blocks(nc);
  const int iters_max = std::max(q->max_iter, 1);
  // rand() draws per iteration in the reference's order: 3 wavelet shifts per cycle spin
  // (L1_threshold, wavelet3D.cpp:443-448), then 3 block shifts per block iteration
  // (LOWRANKCOIL::thresh, which returns before drawing when clear_alpha_coil is 0)
  std::vector<int> sh((size_t)iters_max * 3 * std::max(q->block_iter, 1), 0);
  std::vector<int> wsh((size_t)iters_max * 3 * std::max(q->use_threshold ? q->cycle_spins : 1, 1), 0);
  {
    GlibcRand rng;
    rng.skip(q->rand_skip);
    const int wN = q->wave_type == 0 ? 2 : 4;
    for (int it = 0; it < q->max_iter; it++) {
      if (q->use_threshold)
        for (int sp = 0; sp < q->cycle_spins; sp++)
          for (int d = 0; d < 3; d++) wsh[((size_t)it * q->cycle_spins + sp) * 3 + d] = rng.next() % wN;
      if (q->alpha_coil != 0.0f)
        for (int b = 0; b < q->block_iter; b++)
          for (int d = 0; d < 3; d++) sh[((size_t)it * q->block_iter + b) * 3 + d] = rng.next() % bs[d] - bs[d] / 2;
    }
  }
  int L[3] = {0, 0, 0}, max_level = 0;
  if (q->use_threshold) wavelet_levels(g.N, q->wave_levels, L, &max_level);
  struct Bufs {
    void *p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    ThrWork thr;
    ~Bufs() {
      for (void *x : p) cudaFree(x);
      thr_free(thr);
    }
  } b;
  const size_t sbytes = sizeof(double) * (3 * (size_t)iters_max + 3 * (size_t)nblk + nb + np2) + 2 * sizeof(float) +
                        sizeof(int) * (sh.size() + wsh.size()) + 64;
  MRG_CUDA(cudaMalloc(&b.p[0], sizeof(float2) * ntc));  // XX
  MRG_CUDA(cudaMalloc(&b.p[1], sizeof(float2) * ntc));  // RR
  MRG_CUDA(cudaMalloc(&b.p[2], sizeof(float2) * (nc + n)));  // PP of one frame, unit image
  MRG_CUDA(cudaMalloc(&b.p[3], sbytes));
  float2 *XX = (float2 *)b.p[0], *RR = (float2 *)b.p[1], *PP = (float2 *)b.p[2], *ones = PP + nc;
  double *acc = (double *)b.p[3], *part = acc + 3 * iters_max, *sig = part + 3 * nblk, *work = sig + nb;
  float *smax = (float *)(work + np2), *dthr = smax + 1;
  int *dsh = (int *)(smax + 2), *dwsh = dsh + sh.size();
  MRG_CUDA(cudaMemcpyAsync(dsh, sh.data(), sizeof(int) * sh.size(), cudaMemcpyHostToDevice, st));
  MRG_CUDA(cudaMemcpyAsync(dwsh, wsh.data(), sizeof(int) * wsh.size(), cudaMemcpyHostToDevice, st));
  float2 *W = nullptr;  // frame 0's coil images as C volumes for the wavelet
  if (q->use_threshold) {
    MRG_CUDA(cudaMalloc(&b.p[4], sizeof(float2) * nc));
    W = (float2 *)b.p[4];
    MRG_TRY(thr_alloc(b.thr, nc));
  }
  MRG_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 3 * iters_max, st));
  MRG_TRY(launch_zero(XX, sizeof(float2) * ntc, st));  // XX = 0
  MRG_TRY(launch_fill(ones, n, make_float2(1.0f, 0.0f), st));
  const float *wx = p->d_win + g.og[0], *wy = p->d_win + g.S[0] + g.og[1], *wz = p->d_win + g.S[0] + g.S[1] + g.og[2];
  std::vector<float> diffs;  // residual / residual of iteration 0, for the early stop
  std::vector<double> hacc(3);
  double error0 = 0.0;
  int done = 0;
  for (int it = 0; it < q->max_iter; it++) {
    double *ai = acc + 3 * it;
    for (int t = 0; t < T; t++) {
      const FrameTraj &ft = p->frames[t];
      float2 *Xt = XX + t * nc, *Rt = RR + t * nc;
      // R_c = E_c^H W (E_c X_c - d_c)
      MRG_TRY(run_E(p, ft, ones, Xt, ft.dsorted, p->d_y, true, st));
      MRG_TRY(run_EH_crop(p, ft, p->d_y, st));
      MRG_TRY(launch_coil_images(p->d_t2, C, g.N, wx, wy, wz, Rt, C, 1, false, st));
      // P_c = E_c^H W E_c R_c
      MRG_TRY(run_E(p, ft, ones, Rt, nullptr, p->d_y, true, st));
      MRG_TRY(run_EH_crop(p, ft, p->d_y, st));
      MRG_TRY(launch_coil_images(p->d_t2, C, g.N, wx, wy, wz, PP, C, 1, false, st));
      MRG_TRY(clear_dots(Rt, PP, nc, part, nblk, ai, st));
    }
    MRG_TRY(clear_step(XX, RR, ntc, ai, st));  // XX -= (R^H R / sum P conj R) R
    done = it + 1;
    if (q->use_threshold) {  // L1_threshold(XX(0, all, all)) with cycle spinning (src/recon_lib.cpp:2491-2509)
      MRG_TRY(launch_deinterleave(XX, C, n, W, n, st));
      const float scale = (float)(1. / (float)q->cycle_spins);
      for (int sp = 0; sp < q->cycle_spins; sp++) {
        const int *s3 = dwsh + ((size_t)it * q->cycle_spins + sp) * 3;
        MRG_TRY(wavelet3d(W, C, g.N, L, max_level, s3, q->wave_type, 0, st));
        if (sp == 0) MRG_TRY(fraction_threshold(W, nc, q->thresh, scale, b.thr, dthr, st));
        MRG_TRY(soft_threshold(W, nc, dthr, st));
        MRG_TRY(wavelet3d(W, C, g.N, L, max_level, s3, q->wave_type, 1, st));
      }
      MRG_TRY(launch_interleave(W, n, C, n, XX, st));
    }
    if (q->alpha_coil != 0.0f) {  // lrankcoil.update_threshold(XX, 2, it); lrankcoil.thresh(XX, 2)
      MRG_TRY(coil_llr_update(XX, T, C, g.N, bs, q->clear_amp, q->clear_t2, it, sig, work, smax, st));
      MRG_TRY(coil_llr_thresh(XX, T, C, g.N, bs, q->alpha_coil, q->block_iter, dsh + 3 * (size_t)q->block_iter * it,
                              smax, st));
    }
    if (q->early_stop_range > 0 && q->early_stop_thresh > 0.0f) {  // src/recon_lib.cpp:1118-1125, :1210-1219
      MRG_CUDA(cudaMemcpyAsync(hacc.data(), ai, sizeof(double) * 3, cudaMemcpyDeviceToHost, st));
      MRG_CUDA(cudaStreamSynchronize(st));
      if (it == 0) error0 = hacc[0];
      if (early_stop_met(diffs, (float)(std::fabs(hacc[0]) / error0), q->early_stop_range, q->early_stop_thresh))
        break;
    }
  }
  // lrankcoil.combine(XX, X) into zeroed images
  void *dX;
  bool sX;
  MRG_TRY(dev_view(p, 0, X, sizeof(float2) * n * T, false, st, &dX, &sX));
  MRG_TRY(launch_zero(dX, sizeof(float2) * n * T, st));
  MRG_TRY(coil_combine(XX, T, C, g.N, bs, (float2 *)dX, st));
  if (sX) MRG_CUDA(cudaMemcpyAsync(X, dX, sizeof(float2) * n * T, cudaMemcpyDeviceToHost, st));
  if (coil_images) MRG_CUDA(cudaMemcpyAsync(coil_images, XX, sizeof(float2) * ntc, cudaMemcpyDefault, st));
  if (resid)
    for (int it = 0; it < done; it++)
      MRG_CUDA(cudaMemcpyAsync(resid + it, acc + 3 * it, sizeof(double), cudaMemcpyDeviceToHost, st));
  if (iters) *iters = done;
  p->last_iters = done;
  MRG_CUDA(cudaStreamSynchronize(st));
  return plan_check(p, st);
}

extern "C" {

void mrg_clear_params_default(mrg_clear_params *q) {
  if (!q) return;
  q->max_iter = 50;
  q->block[0] = q->block[1] = q->block[2] = 4;
  q->block_iter = 4;
  q->alpha_coil = 0.01f;
  q->clear_amp = 4.0f;
  q->clear_t2 = 6.0f;
  q->early_stop_thresh = 0.0f;
  q->early_stop_range = 5;
  q->rand_skip = 0;
  q->use_threshold = 0;
  q->thresh = 0.0f;
  q->cycle_spins = 4;
  q->wave_levels[0] = q->wave_levels[1] = q->wave_levels[2] = 4;
  q->wave_type = 1;
}

void mrg_fista_params_default(mrg_fista_params *q) {
  if (!q) return;
  q->max_iter = 50;
  q->max_eig_iter = 30;
  q->fista = 1;
  q->cycle_spins = 4;
  q->wave_levels[0] = q->wave_levels[1] = q->wave_levels[2] = 4;
  q->wave_type = 1;
  q->thresh = 0.0f;
  q->use_threshold = 0;
  q->llr_block[0] = q->llr_block[1] = q->llr_block[2] = 4;
  q->llr_block_iter = 4;
  q->llr_alpha = 0.0f;
  q->clear_amp = 4.0f;
  q->clear_t2 = 6.0f;
  q->rand_skip = -1;
  q->early_stop_thresh = 0.0f;
  q->early_stop_range = 5;
}

mrg_status mrg_set_wait_limit(mrg_plan *p, double seconds) {
  if (!p || !(seconds >= 0.0) || seconds > 3600.0) {
    set_error("wait limit must be within [0, 3600] seconds");
    return MRG_ERR_INVALID;
  }
  p->wait_ns = (long long)(seconds * 1e9);
  invalidate_graphs(p);  // captured launches carry the old limit
  return MRG_OK;
}

mrg_status mrg_plan_check(mrg_plan *p, void *stream) {
  if (!p) {
    set_error("null plan");
    return MRG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  MRG_CUDA(cudaStreamSynchronize(st));
  return plan_check(p, st);
}

mrg_status mrg_last_iterations(const mrg_plan *p, int *iters) {
  if (!p || !iters) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  *iters = p->last_iters;
  return MRG_OK;
}

}  // extern "C"
