// Internal declarations shared by the CUDA translation units of libmrg.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "mrg.h"

namespace mrg {

// ---------------------------------------------------------------------------
// errors and launch accounting
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
extern std::atomic<int64_t> g_launches;
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#define MRG_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) {                                                                    \
      ::mrg::set_error(std::string(#call) + " failed: " + cudaGetErrorString(e_));              \
      return e_ == cudaErrorMemoryAllocation ? MRG_ERR_NOMEM : MRG_ERR_CUDA;                    \
    }                                                                                           \
  } while (0)
#define MRG_LAUNCHED()                                                                          \
  do {                                                                                          \
    ::mrg::count_launch();                                                                      \
    cudaError_t e_ = cudaGetLastError();                                                        \
    if (e_ != cudaSuccess) {                                                                    \
      ::mrg::set_error(std::string("kernel launch failed: ") + cudaGetErrorString(e_));         \
      return MRG_ERR_CUDA;                                                                      \
    }                                                                                           \
  } while (0)
#define MRG_TRY(call)              \
  do {                             \
    mrg_status s_ = (call);        \
    if (s_ != MRG_OK) return s_;   \
  } while (0)

// One-time set-up per device.  Kernel attributes (cudaFuncSetAttribute) and device
// tables belong to the device that is current when they are set, so a process that
// drives several GPUs has to set them once on each; `fn` runs with that device current.
struct DeviceOnce {
  std::mutex mu;
  uint64_t done = 0;  // bit d: set up on device d
};
template <class F>
inline mrg_status device_once(DeviceOnce &o, F &&fn) {
  int dev = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fn();  // beyond the mask: set up on every call
  std::lock_guard<std::mutex> lock(o.mu);
  if ((o.done >> dev) & 1ull) return MRG_OK;
  const mrg_status s = fn();
  if (s == MRG_OK) o.done |= 1ull << dev;
  return s;
}
// Streaming multiprocessors of the current device.
int device_sms();

// Error word of a plan's bounded device-side waits (GridConst::err): 0 while every wait
// ended in time, MRG_WAIT_EXPIRED once one ran out.
constexpr int MRG_WAIT_EXPIRED = 1;
// ... or MRG_REGION_RANGE when a gridding work item named a region outside the grid
constexpr int MRG_REGION_RANGE = 2;
// Default limit of one bounded wait, in nanoseconds of the GPU's global timer.
constexpr long long MRG_DEFAULT_WAIT_NS = 2000000000LL;

// ---------------------------------------------------------------------------
// Geometry: grid sizes, crop, kernel LUT and deapodisation windows, computed on
// the host exactly as gridFFT::precalc_gridding / precalc_kernel do
// (src/gridFFT.cpp:276-643).
// ---------------------------------------------------------------------------
struct Geometry {
  int N[3], S[3], og[3];
  float grid[3], dwin[3], beta[3], grid_mod[3];
  double kb_norm[3];  // the table's normalisation factor (analytic evaluation uses the same scale)
  float k_rad;
  int kernel_type;
  int lut_len;
  std::vector<float> lut[3];
  std::vector<float> win[3];
};
void build_geometry(Geometry &g, const mrg_config &cfg, int Nx, int Ny, int Nz);
// The checks of mrg_plan_create and mrg_plan_geometry: sizes in 1..65536 and options in
// range (overgrid 1..8, dwin -1 or in (0, 16], the enumerations), so that grids and tables
// stay well within int and memory; sets the error text when it returns false.
bool config_ok(const mrg_config &cfg, int Nx, int Ny, int Nz);

// glibc random() stream for the default seed (srand never called by the reference).
struct GlibcRand {
  uint32_t r[34];
  int64_t pos;
  GlibcRand();
  void skip(int64_t n);
  int next();
};

// ---------------------------------------------------------------------------
// Batched strided FFT pass (fft.cu).  A pass transforms `nlines` lines of
// length S; line j = (o, i) with o = j / inner, i = j % inner.  Input row l of
// line (o,i) sits at in[o*in_os + (l - in_off)*in_ls + i] for l in
// [in_off, in_off + Lin) and is zero elsewhere; output rows [out_off,
// out_off + Lout) go to out[o*out_os + (l - out_off)*out_ls + i].
// ---------------------------------------------------------------------------
enum { FFT_PLAIN = 0, FFT_SETIMG = 1, FFT_ACCUM = 2 };
struct FftPass {
  int S, sign, mode;
  int Lin, in_off, Lout, out_off;
  int inner, IB, lfast;
  int vec16, vec16o;  // 16-byte loads / stores of line pairs (set by fft_vectorize)
  int nib;            // inner / IB when no CTA straddles an outer row, else 0 (set by launch_fft)
  int64_t nlines;
  int64_t in_ls, in_os, out_ls, out_os;
  float scale;
  const float2 *in;
  float2 *out;
  const float2 *tw;  // set by launch_fft: exp(-2 pi i m / S)
  // FFT_SETIMG: v = w(l, o, i) * X[off/C] * in[off]  (in = smap or NULL)
  // FFT_ACCUM : acc[l*acc_l + o*acc_o + i/C] += sum_c w(l, o, i)*v*conj(smap[...])
  // w: wmode 0 (lines along z, o = y, i/C = x): (wl[l] * wo[o]) * wi[i/C]
  //    wmode 1 (lines along x, o = z*wdiv + y):  (wo[o / wdiv] * wi[o % wdiv]) * wl[l]
  // both the reference's (winz * winy) * winx
  const float2 *X;
  const float2 *smap;
  float2 *acc;
  const float *wl, *wo, *wi;
  int wmode;
  int64_t wdiv;
  int C, has_smap;
  int acc_atomic;
  int64_t acc_l, acc_o;  // accumulator strides for l and o (i/C has stride 1)
  int xp;                // 1: persistent set_image / accumulate x passes; 2: those and the plain passes with 16 threads
                         // per line; | 4: the plain persistent passes' tiles copied by tensor maps
  int *err;              // device error word (bounded waits of the tensor-map copies; may be NULL)
};
bool fft_size_supported(int S);
// Lines per CTA a pass of length S can take (16 threads per line above 384 points).
int fft_max_lines_per_cta(int S);
// Enables 16-byte line-pair copies when every stride, the line count and the pointers allow it.
void fft_vectorize(FftPass &p);
mrg_status fft_init_device();
mrg_status launch_fft(const FftPass &p, cudaStream_t st);

// ---------------------------------------------------------------------------
// Gridding (gridding.cu)
// ---------------------------------------------------------------------------
// Gridding blocks: one warp owns BLK_X x BLK_Y x BLK_Z grid points (lane = point).
constexpr int BLK_X = 8, BLK_Y = 2, BLK_Z = 2;
static_assert(BLK_X * BLK_Y * BLK_Z == 32, "one grid point per lane");

struct GridConst {
  int S[3];
  float grid[3], cen[3], dwin[3], gmod[3];
  const float *lut[3];
  float k_rad;
  int B;       // sort tile edge (sample order)
  int nt[3];   // sort tiles per axis
  int mbits;   // bits per axis of the tiles' Morton keys
  int nb[3];   // gridding blocks per axis
  int C;       // coils
  int eval;    // 0: table interpolation, 1: analytic Kaiser-Bessel
  int grid_mode;  // 0: fastest timed, 1: CUDA cores, 2: mma.sync tensor cores, 3: tcgen05 / TMEM
  float beta[3];
  double kb_norm[3];
  int *err;          // device word set to MRG_WAIT_EXPIRED when a bounded wait runs out (may be NULL)
  long long wait_ns; // limit of one bounded wait (GPU global timer, ns)
};

// Gridding blocks of b[0] x b[1] x b[2] points, nb[d] = S[d] / b[d] per axis.
struct BlockShape {
  int b[3], nb[3];
};
// Tensor-memory gridding regions: 128 points, one TMEM lane each.
constexpr int RGN_X = 8, RGN_Y = 4, RGN_Z = 4;
static_assert(RGN_X * RGN_Y * RGN_Z == 128, "one region row per TMEM lane");

// A device array that trajectory set-ups reuse: it is reallocated only when a set-up
// needs more bytes than it holds (cap), so repeated set-ups of similar trajectories
// allocate and free nothing (cudaFree waits for the whole device).
template <typename T>
inline mrg_status grow(T *&p, size_t &cap, int64_t n) {
  const size_t want = sizeof(T) * (size_t)(n > 1 ? n : 1);
  if (p && cap >= want) return MRG_OK;
  cudaFree(p);
  p = nullptr;
  cap = 0;
  MRG_CUDA(cudaMalloc((void **)&p, want));
  cap = want;
  return MRG_OK;
}

// (sample, block) pairs of one block shape and the work items over them.
struct PairSet {
  int *pairs = nullptr;     // sample index per (sample, block) pair, grouped by block
  int64_t npairs = 0;
  int4 *items = nullptr;    // (block, p0, p1, split)
  int nitems = 0;
  int *split = nullptr;     // blocks with several work items (pre-zeroed, atomic flush)
  int nsplit = 0;
  bool built = false;       // built for the frame's current trajectory
  size_t cap_pairs = 0, cap_items = 0, cap_split = 0;
};

// Temporaries of a trajectory set-up, kept with the frame for the next one.
struct SetupScratch {
  float4 *pos = nullptr;
  float *tap = nullptr;
  int *key = nullptr, *cnt = nullptr, *off = nullptr, *cur = nullptr;
  int *pcnt = nullptr, *poff = nullptr, *pcur = nullptr, *icnt = nullptr, *ioff = nullptr, *nsplit = nullptr;
  size_t cap_pos = 0, cap_tap = 0, cap_key = 0, cap_cnt = 0, cap_off = 0, cap_cur = 0;
  size_t cap_pcnt = 0, cap_poff = 0, cap_pcur = 0, cap_icnt = 0, cap_ioff = 0, cap_nsplit = 0;
};

struct FrameTraj {
  int64_t M = 0;
  int nvalid = 0;
  float4 *spos = nullptr;   // [M] sorted, valid first: (dkx, dky, dkz, kw)
  float *stap = nullptr;    // [M] taper exp(-|k|^2/(2 k_rad^2))
  float *skr = nullptr;     // [M] |k|^2 (float, as the reference sums it), for a new k_rad
  int *perm = nullptr;      // [M] sorted -> original sample index
  float4 *swt = nullptr;    // [nvalid][6] tap weights wx[8], wy[8], wz[8] (chop sign included, zero padded)
  int4 *sst = nullptr;      // [nvalid] first tap (sx, sy, sz) and tap counts nx | ny << 4 | nz << 8
  PairSet blocks;           // 8x2x2 blocks (k_grid, k_grid_mma)
  PairSet regions;          // 8x4x4 regions (k_grid_umma), built when that kernel may run
  // per 96-pair chunk of the region work items: (wz*wy) for the region's 16 (z, y) rows and
  // wx for its 8 x, 24 rows x 100 floats (k_grid_umma's shared-memory layout); rchunk[item]
  // = the item's first chunk (items without pairs have none)
  float *rtab = nullptr;
  int *rchunk = nullptr;
  int64_t nrchunks = 0;
  float2 *dsorted = nullptr;  // measured data [nvalid][C], unweighted
  float4 *sdw = nullptr;      // [nvalid][6] d(tap weight)/dk per axis (allocated by mrg_grad)
  bool has_data = false;
  bool sdw_valid = false;     // sdw computed for the current trajectory
  // bytes held by each array above (reused by the next set-up of this frame)
  size_t cap_spos = 0, cap_stap = 0, cap_skr = 0, cap_perm = 0, cap_swt = 0, cap_sst = 0, cap_rtab = 0,
         cap_rchunk = 0, cap_dsorted = 0, cap_sdw = 0;
  SetupScratch scr;
  // launch shapes picked by autotune_frame (0: defaults)
  int ungrid_G = 0, ungrid_spb = 0, ungrid_cpl = 0, ungrid_uy = 0, grid_cc = 0;
  float tune_ungrid_ms = 0.f, tune_grid_ms = 0.f;
};

// The 8x2x2 block pair lists of the CUDA-core and mma.sync gridding kernels (once per trajectory).
mrg_status build_block_pairs(const GridConst &gc, FrameTraj &ft, int max_pairs, cudaStream_t st);
mrg_status traj_setup(const GridConst &gc, FrameTraj &ft, const float *kx, const float *ky, const float *kz,
                      const float *kw, int64_t M, int max_pairs, bool regions, cudaStream_t st);
BlockShape block_shape(const GridConst &gc);
BlockShape region_shape(const GridConst &gc);
void pair_set_free(PairSet &ps);
// tcgen05 gridding over 8x4x4 regions (grid_umma.cu): cc = coils per pass (8, 16 or 32)
bool umma_supported(int C);
bool umma_grid_fits(const int S[3]);
// Packs the region origin into each work item of the tcgen05 kernel's pair set.
mrg_status pack_region_items(const GridConst &gc, PairSet &ps, cudaStream_t st);
// The region tables of ft.regions (ft.rtab, ft.rchunk), after pack_region_items.
mrg_status build_region_tables(FrameTraj &ft, cudaStream_t st);
// its pieces (grid_umma.cu): chunks per work item into cnt[], and the tables themselves
int64_t umma_table_floats();  // floats per chunk
mrg_status launch_item_chunks(const FrameTraj &ft, int *cnt, cudaStream_t st);
mrg_status launch_region_tables(const FrameTraj &ft, cudaStream_t st);
// a gridding launch shape (mrg_frame_tuning's encoding) that the frame's kernels can run
bool grid_cc_allowed(int C, const FrameTraj &ft, int cc);
// n-tiles (4 coils each) per pass of the tensor-core ungridding kernel; 0: needs C % 4 == 0
int ungrid_mma_nt(int C);
int umma_default_cc(int C);
mrg_status launch_grid_umma(const GridConst &gc, const FrameTraj &ft, int cc, const float2 *yw, float2 *grid,
                            cudaStream_t st);
// the error word gc.err (0 when gc.err is NULL); reading it waits for the device
int read_wait_error(const GridConst &gc);
void traj_free(FrameTraj &ft);
mrg_status launch_retaper(const GridConst &gc, FrameTraj &ft, cudaStream_t st);
mrg_status count_taps(const FrameTraj &ft, int64_t *out);
// coil images / sum of squares from the cropped E^H transform t[v][c]; blur; SOS normalisation
mrg_status launch_coil_images(const float2 *t, int C, const int N[3], const float *wx, const float *wy,
                              const float *wz, float2 *out, int64_t es, int64_t vs, bool accumulate,
                              cudaStream_t st);
mrg_status launch_sos_images(const float2 *t, int C, const int N[3], const float *wx, const float *wy,
                             const float *wz, float2 *X, cudaStream_t st);
mrg_status gaussian_blur_ex(float2 *X, int nvol, const int N[3], int64_t es, int64_t vs, const float sigma[3],
                            cudaStream_t st);
mrg_status sos_normalize_ex(float2 *A, int C, int64_t nimg, int64_t es, int64_t vs, cudaStream_t st);
// Pipe density compensation on device trajectories (dcf.cu)
mrg_status dcf_pipe(const float *kx, const float *ky, const float *kz, int64_t M, const int N[3], int iters,
                    float dwin, float scale, float overgrid, float acc, int kernel, float *kw, cudaStream_t st);
// y[s][c] = sum over taps of grid (gridFFT::chop_grid_backward), minus diff[s][c] if given;
// with `weigh` the result is multiplied by kw and the taper, ready for launch_grid.
mrg_status launch_ungrid(const GridConst &gc, const FrameTraj &ft, const float2 *grid, const float2 *diff,
                         float2 *y, bool weigh, cudaStream_t st);
// grid = scatter of the already weighted samples yw (gridFFT::chop_grid_forward); every point written.
mrg_status launch_grid(const GridConst &gc, const FrameTraj &ft, const float2 *yw, float2 *grid, cudaStream_t st);
// d(weights)/dk per sample (analytic Kaiser-Bessel derivative), for mrg_grad.
mrg_status launch_sample_dweights(const GridConst &gc, FrameTraj &ft, cudaStream_t st);
// Per sample: v = E x (from the grid), r = v - ysorted; writes 2r over ysorted, grad_k
// (user order, [3][M]) and adds sum |r|^2 (and sum |y|^2 of the non-contributing samples
// read from the user's y) into *loss.
mrg_status launch_ungrid_grad(const GridConst &gc, const FrameTraj &ft, const float2 *grid, float2 *ysorted,
                              const float2 *y_user, int64_t stride, float *grad_k, double *loss, cudaStream_t st);
// Times the candidate launch shapes of the ungridding and gridding kernels for this
// frame on the given buffers and stores the fastest in `ft`.
mrg_status autotune_frame(const GridConst &gc, FrameTraj &ft, float2 *grid, float2 *y, cudaStream_t st);
// dst[s][c] = src[c*stride + perm[s]] (times kw*taper with `weigh`), s < nvalid
mrg_status launch_gather_samples(const FrameTraj &ft, int C, const float2 *src, int64_t stride, float2 *dst,
                                 cudaStream_t st, bool weigh = false);
// dst[s][c] = src[s][c] * kw * taper
mrg_status launch_weigh_samples(const FrameTraj &ft, int C, const float2 *src, float2 *dst, cudaStream_t st);
// dst[c*stride + perm[s]] = s < nvalid ? src[s][c] : 0
mrg_status launch_scatter_samples(const FrameTraj &ft, int C, const float2 *src, float2 *dst, int64_t stride,
                                  cudaStream_t st);

// ---------------------------------------------------------------------------
// Vector kernels (solver.cu)
// ---------------------------------------------------------------------------
struct Scalars {
  double rr, rn, e;
  double pl[2];
  float alpha[2], beta[2];
  float step;
  int it;
  int pad;
};
mrg_status launch_interleave(const float2 *src, int64_t stride, int C, int64_t n, float2 *dst, cudaStream_t st);
mrg_status launch_deinterleave(const float2 *src, int C, int64_t n, float2 *dst, int64_t stride, cudaStream_t st);
mrg_status launch_zero(void *p, size_t bytes, cudaStream_t st);
// dst (device) <- bytes of pinned host memory addressed through its device-side alias src
mrg_status launch_copy_from_host(void *dst, const void *src, size_t bytes, cudaStream_t st);
mrg_status launch_copy(float2 *dst, const float2 *src, int64_t n, cudaStream_t st);
mrg_status cg_dots(const float2 *R, const float2 *P, const float2 *L, int64_t n, double *part, int nblk,
                   Scalars *sc, cudaStream_t st);
mrg_status cg_update(float2 *X, float2 *R, const float2 *P, const float2 *L, int64_t n, double *part, int nblk,
                     Scalars *sc, double *resid, cudaStream_t st);
mrg_status cg_pupdate(float2 *P, const float2 *R, int64_t n, const Scalars *sc, cudaStream_t st);
int reduce_blocks(int64_t n);
// Blocks for a grid-stride loop over n items: enough to fill the 152 SMs many times over.
inline int grid_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 64) b = 152 * 64;
  return (int)b;
}

// FISTA pieces
mrg_status launch_fill(float2 *X, int64_t n, float2 v, cudaStream_t st);
mrg_status energy(const float2 *R, int64_t n, double *part, int nblk, double *out, cudaStream_t st);
mrg_status power_scale(float2 *X, const float2 *R, int64_t n, Scalars *sc, cudaStream_t st);
mrg_status fista_momentum(float2 *X, float2 *Xo, int64_t n, const Scalars *sc, int fista, cudaStream_t st);
mrg_status grad_step(float2 *X, const float2 *R, int64_t n, const Scalars *sc, double *part, int nblk,
                     double *resid, cudaStream_t st);
mrg_status bump_iteration(Scalars *sc, cudaStream_t st);

// wavelet.cu (shifts[(sc ? sc->it : 0) * per_it + off + axis])
mrg_status wavelet3d_ex(float2 *X, int nvol, const int N[3], const int L[3], int max_level, const int *shifts,
                        const Scalars *sc, int per_it, int off, int wave_type, int inverse, cudaStream_t st);
mrg_status wavelet3d(float2 *X, int nvol, const int N[3], const int L[3], int max_level, const int *shifts_dev,
                     int wave_type, int inverse, cudaStream_t st);
void wavelet_levels(const int N[3], const int levels_in[3], int L[3], int *max_level);

// threshold.cu
struct ThrWork {
  float *mag = nullptr;
  unsigned long long *cnt = nullptr;
  float *state = nullptr;  // value, min_t, max_t, done
  double *dstate = nullptr;
  int64_t cap = 0;
};
mrg_status thr_alloc(ThrWork &w, int64_t n);
void thr_free(ThrWork &w);
// value written to *out_dev (device float), scaled by `scale`
mrg_status fraction_threshold(const float2 *X, int64_t n, float fraction, float scale, ThrWork &w, float *out_dev,
                              cudaStream_t st);
mrg_status soft_threshold(float2 *X, int64_t n, const float *value_dev, cudaStream_t st);

// llr.cu
struct LlrWork {
  double *sig = nullptr;
  float *smax = nullptr;
  int nb = 0;
};
mrg_status llr_alloc(LlrWork &w, int nblocks);
void llr_free(LlrWork &w);
mrg_status llr_update(const float2 *X, int Nt, const int N[3], const int bs[3], float amp, float t2,
                      const int *iter_dev, LlrWork &w, cudaStream_t st);
// Blocks of bs[0] x bs[1] x bs[2] voxels (clipped to N) that tile N; 64-bit, so callers can
// reject counts their buffers and launches cannot take.
int64_t llr_block_count(const int N[3], const int bs[3]);
// sigma_1 of every block into sig[nblocks], median via work[next pow2 >= nblocks], result in *smax (device).
mrg_status llr_update_into(const float2 *X, int Nt, const int N[3], const int bs[3], float amp, float t2,
                           const Scalars *sc, int iter_fixed, double *sig, double *work, float *smax, cudaStream_t st);
mrg_status llr_update_ex(const float2 *X, int Nt, const int N[3], const int bs[3], float amp, float t2,
                         const Scalars *sc, int iter_fixed, LlrWork &w, cudaStream_t st);
// Median of the n non-zero sigma_1 in sig (work: next power of two doubles) times
// (1 + amp exp(-iter / t2)) into the device float smax.
mrg_status llr_median(const double *sig, int n, double *work, float amp, float t2, int iter, float *smax,
                      cudaStream_t st);
// ESPIRiT maps from coil images [voxel][coil] (espirit.cu)
struct EspiritParams {
  float kr_f[3];
  int cr[3];
  float svd_thresh;
  int square;
  double *sv_out;  // host, may be NULL: calibration singular values, descending
  int sv_cap;
};
mrg_status espirit_maps(const float2 *img, int C, const int N[3], const EspiritParams &q, float2 *maps, int *nV_out,
                        cudaStream_t st);
// CLEAR coil low rank on [frame][voxel][coil] stacks (clear.cu)
int64_t coil_llr_blocks(const int N[3], const int bs[3]);
mrg_status coil_llr_update(const float2 *X, int T, int C, const int N[3], const int bs[3], float amp, float t2,
                           int iter, double *sig, double *work, float *smax, cudaStream_t st);
mrg_status coil_llr_thresh(float2 *X, int T, int C, const int N[3], const int bs[3], float alpha, int block_iter,
                           const int *shifts, const float *smax, cudaStream_t st);
mrg_status coil_combine(const float2 *X, int T, int C, const int N[3], const int bs[3], float2 *out,
                        cudaStream_t st);
// CLEAR gradient step: acc[0..2] += (sum |R|^2, sum P conj(R)); X -= (acc0 / acc12) R
mrg_status clear_dots(const float2 *R, const float2 *P, int64_t n, double *part, int nblk, double *acc,
                      cudaStream_t st);
mrg_status clear_step(float2 *X, const float2 *R, int64_t n, const double *acc, cudaStream_t st);
mrg_status llr_apply_ex(float2 *X, int Nt, const int N[3], const int bs[3], int block_iter, float alpha,
                        const int *shifts, const Scalars *sc, int per_it, int off_base, const float *smax_dev,
                        cudaStream_t st);
mrg_status llr_apply(float2 *X, int Nt, const int N[3], const int bs[3], int block_iter, float alpha,
                     const int *shifts_dev, const float *smax_dev, cudaStream_t st);

}  // namespace mrg
