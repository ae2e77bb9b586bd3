/*
 * mrg.h -- C ABI of the GB300-native gridFFT / SENSE hot path.
 *
 * One plan replaces one uwmri/mri_recon `gridFFT` operator (src/gridFFT.h:28-194)
 * together with the coil-batched `gridFFT_CoilThreaded` (src/gridFFT_CoilThreaded.h:26-191)
 * and the CG / FISTA loops of `RECON::full_recon` (src/recon_lib.cpp:1523-2212) that drive
 * them.  Every entry point returns an mrg_status and never exits the process (the
 * reference calls exit(1), e.g. src/ArrayTemplates.cpp:290-293).
 *
 * Naming: the reference calls E^H (k-space -> image) `gridFFT::forward` and E
 * (image -> k-space) `gridFFT::backward`.  Here mrg_adjoint* is E^H and mrg_forward*
 * is E; each declaration names the reference function it replaces.
 *
 * Layouts follow the reference's Blitz arrays: images are complex64 [Nz][Ny][Nx]
 * (x fastest, column-major in Blitz terms), k-space samples are flat complex64 arrays
 * of M samples (the readout x projection x slice arrays of src/mri_data.h, flattened
 * readout-fastest), trajectories are float32 arrays in the reference's units
 * (k in [-N/2, N/2], src/commandline_recon.cxx:68-72).
 *
 * Pointers may be device pointers or host pointers; host buffers are staged through
 * device memory inside the call.  `stream` is a cudaStream_t (NULL = legacy default).
 * A plan is not re-entrant: calls on one plan must be serialised on one stream, as the
 * reference's shared k3d_grid makes one gridFFT instance non-re-entrant.
 */
#ifndef MRG_H
#define MRG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mrg_plan mrg_plan;

typedef enum mrg_status {
  MRG_OK = 0,
  MRG_ERR_INVALID = 1,     /* bad argument or shape */
  MRG_ERR_CUDA = 2,        /* CUDA runtime error (message in mrg_last_error) */
  MRG_ERR_NOMEM = 3,       /* device allocation failed */
  MRG_ERR_STATE = 4,       /* call out of order (e.g. no trajectory set) */
  MRG_ERR_TIMEOUT = 5,     /* a bounded device-side wait ran out (see mrg_set_wait_limit) */
  MRG_ERR_UNSUPPORTED = 6  /* grid size or option this build does not implement */
} mrg_status;

/* gridFFT kernel types (src/gridFFT.h:19-22) */
enum { MRG_KERNEL_TRIANGLE = 0, MRG_KERNEL_KAISER = 1, MRG_KERNEL_SINC = 2, MRG_KERNEL_POLY = 3 };

/* Operator options; the gridFFT public fields set before precalc_gridding
 * (src/gridFFT.cpp:28-60 defaults, :187-245 command-line flags). */
typedef struct mrg_config {
  float overgrid;    /* gridFFT::overgrid, -overgrid (default 1.5) */
  float dwin;        /* gridFFT::dwinX/Y/Z, -dwinX (-1: kernel default, 2.5 for Kaiser) */
  int kernel_type;   /* gridFFT::kernel_type, -kaiser/-triangle/-sinc/-poly_kernel */
  float k_rad;       /* gridFFT::k_rad, Gaussian taper radius of E^H (default 9999) */
  int time_grid;     /* gridFFT::time_grid, -time_grid: print per-stage device times */
  int tile;          /* sample-sort tile edge in grid points, tiles in Morton order (0: default 2 and
                        autotuned launch shapes; > 0: this edge and fixed launch shapes) */
  int max_pairs;     /* (sample, block) pairs per gridding work item (0: default) */
  int kernel_eval;   /* 0: interpolate the 600-per-unit table as the reference (src/gridFFT.cpp:1113-1116);
                        1: evaluate the Kaiser-Bessel kernel analytically (same beta and scale), the
                        form whose derivative mrg_grad uses, for finite-difference-consistent gradients */
  int grid_mode;     /* gridding (E^H scatter) kernel: 0 the fastest of 1, 2 and 3 (timed per frame),
                        1 FP32 multiply-adds on the CUDA cores, 2 tensor cores through mma.sync, 3
                        tensor cores through tcgen05 with W and the accumulators in tensor memory
                        (>= 8 coils); 2 and 3 in TF32 with the three-term hi/lo split
                        (W V ~ Wh Vh + Wh Vl + Wl Vh, products to ~2^-20) */
  int fft_norm;      /* 0: every FFT pass scaled by 1/sqrt(S), as gridFFT's fft3 (src/ArrayTemplates.cpp:311,
                        :338-342); 1: unnormalised passes, as gridFFT_CoilThreaded's do_fft / do_ifft
                        (src/gridFFT_CoilThreaded.cpp:570-893), so E and E^H (and mrg_fft3) are
                        sqrt(Sx Sy Sz) times those of 0 */
} mrg_config;

/* Fills the reference defaults (src/gridFFT.cpp:28-60). */
void mrg_config_default(mrg_config *cfg);

/* Text of the last error on this thread ("" when none). */
const char *mrg_last_error(void);

/* Replaces gridFFT::precalc_gridding(Nz, Ny, Nx, data) (src/gridFFT.cpp:475-643) for a
 * 3D non-Cartesian trajectory, and gridFFT_CoilThreaded::precalc_gridding for ncoil
 * coils (src/gridFFT_CoilThreaded.cpp:403-568).  nframes trajectories (gated frames /
 * encodes, src/recon_lib.cpp:675-776) can be set on one plan. */
mrg_status mrg_plan_create(const mrg_config *cfg, int Nx, int Ny, int Nz, int ncoil, int nframes, mrg_plan **out);
mrg_status mrg_plan_destroy(mrg_plan *plan);

/* Geometry as computed by precalc_gridding: grid size S (Sx,Sy,Sz), crop start og_s
 * (src/gridFFT.cpp:536-541), grid ratio grid_x/y/z, Kaiser beta, kernel half width and
 * LUT length (src/gridFFT.cpp:330-340). */
mrg_status mrg_plan_info(const mrg_plan *plan, int S[3], int og[3], float grid[3], float beta[3], float dwin[3],
                         int *lut_len);
/* Host copies of the kernel lookup tables grid_filterX/Y/Z (3*lut_len floats) and the
 * deapodisation windows winx, winy, winz (Sx+Sy+Sz floats), src/gridFFT.cpp:276-631. */
mrg_status mrg_get_tables(const mrg_plan *plan, float *lut, float *win);

/* Coil sensitivity maps: ncoil complex64 images, coil c at smaps + c*coil_stride
 * (elements).  Replaces the `smaps` container passed to every forward/backward call
 * (src/recon_lib.cpp:1560-1621). */
mrg_status mrg_set_smaps(mrg_plan *plan, const void *smaps, int64_t coil_stride, void *stream);

/* Trajectory and per-sample weight of one frame: kx, ky, kz, kw of M samples.  kw is
 * the density compensation times the frame's gating weight (the reference's
 * TimeWeight, src/recon_lib.cpp:1543-1557).  Samples with kw == 0 or outside the grid
 * contribute nothing (src/gridFFT.cpp:1035-1098). */
mrg_status mrg_set_traj(mrg_plan *plan, int frame, const float *kx, const float *ky, const float *kz,
                        const float *kw, int64_t M, void *stream);

/* Sample bookkeeping of one frame after mrg_set_traj: M samples, nvalid of them
 * contribute (kw != 0 and inside the grid), npairs (sample, block) pairs and nitems
 * gridding work items of the 8x2x2 block lists (of the 8x4x4 region lists of the tcgen05
 * kernel when the block lists are not built: a plan tuned to that kernel skips them on
 * later trajectories), and ntaps grid points read by one ungridding (the sum of every
 * valid sample's nx*ny*nz; computed on the device when ntaps is not NULL).  Any output
 * may be NULL. */
mrg_status mrg_frame_info(const mrg_plan *plan, int frame, int64_t *M, int64_t *nvalid, int64_t *npairs,
                          int64_t *nitems, int64_t *ntaps);

/* Launch shapes the autotuner chose for a frame (mrg_config.tile == 0): out = {ungrid lanes
 * per sample (-n: the tensor-core kernel, 16 samples per warp, 4n coils per pass), ungrid
 * samples per CTA, gridding coils per pass (0: all; -n with n < 100: the
 * mma.sync kernel with 4n coils per pass; -(100 + c): the tcgen05 kernel with c coils per
 * pass), ungrid coils per lane, ungrid tap rows loaded per step};
 * ms = the timed ungrid and grid kernels. */
mrg_status mrg_frame_tuning(const mrg_plan *plan, int frame, int out[5], float ms[2]);
/* Fixes a frame's launch shapes (same order and encoding as mrg_frame_tuning) after
 * mrg_set_traj, in place of the autotuner's: for reproducible launches or to compare
 * variants.  Gridding shapes the plan cannot run are rejected (MRG_ERR_INVALID); an
 * ungridding shape a buffer cannot take falls back to fewer coils per lane (4 coils per
 * lane needs a coil count divisible by 4 and 4 to 16 lanes; 2 needs an even count). */
mrg_status mrg_frame_set_tuning(mrg_plan *plan, int frame, const int in[5]);
/* FFT launch shapes of the plan (no counterpart in the reference, whose FFTW plans are
 * opaque): per pass k (0-2: E's x/set_image, z, y; 3-5: E^H's y, z, x/accumulate) the
 * lines per CTA ib[k] (0: the default, a multiple of the coil count up to 32) and xp[k] (1:
 * the persistent set_image / accumulate kernel of the x passes of multi-coil plans, used
 * where the pass's strides allow it; 2: the same with 16 threads per line, for lines of
 * 288, 320 and 384 points, which also applies to the persistent plain y and z passes;
 * | 4: the plain persistent passes' tiles copied by tensor maps, TMA).  The first mrg_set_traj of a plan tunes them by
 * timing; mrg_set_fft_tuning fixes them afterwards (values a pass cannot take fall back
 * to its default).  Either array may be NULL. */
mrg_status mrg_fft_tuning(const mrg_plan *plan, int ib[6], int xp[6]);
mrg_status mrg_set_fft_tuning(mrg_plan *plan, const int ib[6], const int xp[6]);

/* Measured k-space of one frame: ncoil arrays of M complex64, coil c at
 * data + c*coil_stride.  Used by mrg_cg / mrg_fista (data.kdata, src/mri_data.h). */
mrg_status mrg_set_data(mrg_plan *plan, int frame, const void *data, int64_t coil_stride, void *stream);

/* E^H, all coils of a frame: X += sum_c gridFFT::forward(X, smap_c, data_c, k, kw)
 * (src/gridFFT.cpp:791-812; coil-batched src/gridFFT_CoilThreaded.cpp:999-1031). */
mrg_status mrg_adjoint(mrg_plan *plan, int frame, const void *data, int64_t coil_stride, void *X, void *stream);

/* E, all coils of a frame: data_c = gridFFT::backward(X, smap_c) (src/gridFFT.cpp:824-844),
 * or data_c = E_c X - diff_c when diff is not NULL (backward_residual,
 * src/gridFFT.cpp:856-876). */
mrg_status mrg_forward(mrg_plan *plan, int frame, const void *X, void *data, int64_t coil_stride, const void *diff,
                       void *stream);

/* out = sum_c E_c^H W E_c X for one frame (the operator of the CG loop,
 * src/recon_lib.cpp:1614-1622).  out is overwritten. */
mrg_status mrg_normal(mrg_plan *plan, int frame, const void *X, void *out, void *stream);

/* Per-coil calls with an explicit sensitivity map, the exact per-coil surface of
 * gridFFT::forward / backward / backward_residual (src/gridFFT.h:109-164).  Valid on a
 * plan created with ncoil == 1; smap may be NULL (the no-smap overloads,
 * src/gridFFT.cpp:759-789 and :887-906). */
mrg_status mrg_adjoint_coil(mrg_plan *plan, int frame, const void *smap, const void *data, void *X, void *stream);
mrg_status mrg_forward_coil(mrg_plan *plan, int frame, const void *X, const void *smap, void *data, const void *diff,
                            void *stream);

/* gridFFT::do_fft / do_ifft (src/gridFFT.cpp:645-711) on a caller grid, unpruned: grid is
 * Sz x Sy x Sx x ncoil complex64 (coil innermost, host or device), transformed in place
 * along z, y, x (sign -1, FFTW_FORWARD) or x, y, z (sign +1, FFTW_BACKWARD), each axis
 * scaled by 1/sqrt(S) (src/ArrayTemplates.cpp:276-427).  The operators run the same
 * passes pruned to the image crop; this entry exposes them for cross-checks. */
mrg_status mrg_fft3(mrg_plan *plan, void *grid, int sign, void *stream);

/* gridFFT::chop_grid_forward / chop_grid_backward (src/gridFFT.cpp:1009-1164, :1166-1322;
 * src/gridFFT.h:177-186) on a caller grid, all coils of a frame, as RECON::kspace_residual
 * calls them on the public k3d_grid (src/recon_lib.cpp:2218-2252).  The grid is
 * Sz x Sy x Sx x ncoil complex64, coil innermost (for one coil the reference's
 * column-major k3d_grid), host or device; the chop sign (-1)^l of every tap is part of the
 * weights, as in the reference.
 *   mrg_grid:   grid = scatter of data_c * kw * taper (the whole grid is written: the
 *               reference's caller zeroes k3d_grid first, then chop_grid_forward adds);
 *   mrg_ungrid: data_c = sum over the taps of grid_c, or that minus diff_c (diff may be NULL). */
mrg_status mrg_grid(mrg_plan *plan, int frame, const void *data, int64_t coil_stride, void *grid, void *stream);
mrg_status mrg_ungrid(mrg_plan *plan, int frame, const void *grid, void *data, int64_t coil_stride, const void *diff,
                      void *stream);

/* The public gridFFT::k_rad field (src/gridFFT.h:102; default 9999): the radius of the
 * Gaussian taper exp(-|k|^2 / (2 k_rad^2)) E^H applies to each sample
 * (src/gridFFT.cpp:1096-1108).  The coil-map estimate sets it to the map resolution and
 * back (src/recon_lib.cpp:2738, :2786).  Applies to every frame's trajectory. */
mrg_status mrg_set_k_rad(mrg_plan *plan, float k_rad, void *stream);

/* Map-free adjoints over all coils of the plan (data coil c at data + c*coil_stride):
 *   mrg_adjoint_coils: images[c*image_stride + v] += E^H_c (kw * data_c), one image per
 *     coil -- gridFFT::forward without a map (src/gridFFT.cpp:759-789, accumulate(X)
 *     :943-958), as the coil-map estimate calls it per coil (src/recon_lib.cpp:2771-2782).
 *   mrg_adjoint_sos: X[v] += sum_c |deapp(E^H_c (kw * data_c))|^2 -- gridFFT::forward_sos
 *     (src/gridFFT.cpp:722-757, accumulate_sos :960-970) summed over coils. */
mrg_status mrg_adjoint_coils(mrg_plan *plan, int frame, const void *data, int64_t coil_stride, void *images,
                             int64_t image_stride, void *stream);
mrg_status mrg_adjoint_sos(mrg_plan *plan, int frame, const void *data, int64_t coil_stride, void *X, void *stream);

/* The default (LOWRES, SOS-normalised) coil-map estimate of RECON::calc_sensitivity_maps
 * (src/recon_lib.cpp:2694-2950 with coil_combine_type LOWRES, smap_norm SOS, smap_thresh 0,
 * one encode): per coil E^H without maps at k_rad = smap_res (flag -smap_res, default 8),
 * a Gaussian blur of sigma blur[3] (flags -extra_blur, default 0: none; may be NULL), then
 * every coil divided by the root sum of squares over coils.  The maps become the plan's
 * maps (as mrg_set_smaps); smaps_out (may be NULL) receives them, coil c at
 * smaps_out + c*out_stride.  k_rad is restored afterwards. */
mrg_status mrg_lowres_smaps(mrg_plan *plan, int frame, const void *data, int64_t coil_stride, float smap_res,
                            const float blur[3], void *smaps_out, int64_t out_stride, void *stream);

/* ESPIRiT coil maps (SPIRIT::generateEigenCoils, src/spirit.cpp:137-550; the ESPIRIT
 * branch of calc_sensitivity_maps, src/recon_lib.cpp:2892-2899).  Fields are the -sp_*
 * flags (-sp_kr_f / -sp_cr set all three axes). */
typedef struct mrg_espirit_params {
  float kernel_radius[3]; /* -sp_krx_f/-sp_kry_f/-sp_krz_f (default 3), at most 7 */
  int calib_radius[3];    /* -sp_crx/-sp_cry/-sp_crz (default 12); must exceed ceil(kernel_radius) */
  float svd_thresh;       /* -sp_svd_thresh (default 0.01): keep s >= s0 sqrt(svd_thresh) */
  int square;             /* -sp_square (1) or -sp_circle (0, default) regions */
} mrg_espirit_params;

void mrg_espirit_params_default(mrg_espirit_params *p);

/* Maps from caller coil images: images and maps are Nx*Ny*Nz voxels x ncoil complex64,
 * coil innermost (host or device).  kept (may be NULL): kernel vectors kept; sv (host,
 * may be NULL): the first sv_cap calibration singular values, descending.  ncoil <= 32. */
mrg_status mrg_espirit(const void *images, int ncoil, int Nx, int Ny, int Nz, const mrg_espirit_params *params,
                       void *maps, int *kept, double *sv, int sv_cap, void *stream);
/* ESPIRiT maps of a plan: the map-free E^H of each coil of `frame` (the plan's k_rad as
 * set: the reference leaves the taper off for ESPIRiT), the optional Gaussian blur
 * (extra_blurX/Y/Z, NULL for none), then mrg_espirit; the maps become the plan's maps and
 * are also written to smaps_out (may be NULL; coil c at smaps_out + c*out_stride). */
mrg_status mrg_espirit_smaps(mrg_plan *plan, int frame, const void *data, int64_t coil_stride,
                             const mrg_espirit_params *params, const float blur[3], void *smaps_out,
                             int64_t out_stride, int *kept, void *stream);

/* SENSE conjugate gradient (src/recon_lib.cpp:1523-1759): X (nframes images) is
 * overwritten with the result of max_iter iterations from x0 = 0, FP32 vectors and
 * FP64 scalars.  resid (host, may be NULL) receives sum|r|^2 after each iteration.
 * use_graph != 0 captures one iteration as a CUDA graph and replays it. */
mrg_status mrg_cg(mrg_plan *plan, int max_iter, void *X, double *resid, int use_graph, void *stream);

/* Differentiable E (no counterpart in the reference; its operator is gridFFT::backward,
 * src/gridFFT.cpp:824-844, with unit density weights), Kaiser-Bessel plans only (other
 * kernels return MRG_ERR_UNSUPPORTED): for one frame
 *   loss   = sum_c || E_c(x, k) - y_c ||^2                     (host double, may be NULL)
 *   grad_x = 2 sum_c E_c^* (E_c x - y_c)  complex64 image       (the exact adjoint, no kw or taper)
 *   grad_k = dloss/dk as float32 [3][M] (kx, ky, kz rows) in the reference's k units,
 * from the analytic derivative of the Kaiser-Bessel kernel.  kw of the frame only selects
 * samples (kw == 0 or outside the grid: E is 0 there and grad_k is 0).  With
 * kernel_eval = 0 the forward interpolates the table while the derivative is analytic (they
 * differ at the table's resolution); kernel_eval = 1 makes both analytic.
 * y: ncoil arrays of M complex64, coil c at y + c*coil_stride. */
mrg_status mrg_grad(mrg_plan *plan, int frame, const void *X, const void *y, int64_t coil_stride, double *loss,
                    void *grad_x, float *grad_k, void *stream);

/* The same loop in three calls, for callers that time or interleave iterations:
 * mrg_cg_init sets X = 0, R = P = sum_c E^H W d (src/recon_lib.cpp:1537-1573) and reserves
 * room for max_iter residuals; mrg_cg_iterate runs n more iterations; mrg_cg_residuals
 * copies the first n residuals to the host.  X must be device memory here. */
mrg_status mrg_cg_init(mrg_plan *plan, int max_iter, void *X, void *stream);
mrg_status mrg_cg_iterate(mrg_plan *plan, int n, void *X, int use_graph, void *stream);
mrg_status mrg_cg_residuals(mrg_plan *plan, double *resid, int n, void *stream);

/* FISTA / IST with L1-wavelet fraction thresholding and optional locally-low-rank
 * thresholding in time (src/recon_lib.cpp:1761-2212, :2416-2527; src/threshold.cpp;
 * src/wavelet3D.cpp; src/clear.cpp:233-556). */
typedef struct mrg_fista_params {
  int max_iter;          /* -max_iter */
  int max_eig_iter;      /* max_eigen_iterations (default 30) */
  int fista;             /* 1 FISTA, 0 IST */
  int cycle_spins;       /* -cycle_spins (default 4) */
  int wave_levels[3];    /* -wavelet_levelsX/Y/Z (default 4) */
  int wave_type;         /* 0 DB2, 1 DB4 (-wavelet_type, default DB4) */
  float thresh;          /* -thresh: fraction of coefficients set to zero (fraction), or the
                            threshold value (fixed) */
  int use_threshold;     /* -threshold_type: none (0), fraction (1) or fixed (2) */
  int llr_block[3];      /* -clear_nx/ny/nz (default 4) */
  int llr_block_iter;    /* -clear_block_iter (default 4) */
  float llr_alpha;       /* -clear_alpha_time (0: off) */
  float clear_amp;       /* -clear_amp (default 4) */
  float clear_t2;        /* -clear_t2 (default 6) */
  int64_t rand_skip;     /* rand() draws consumed before the first shift; -1: the
                            2*N^3*nframes draws of the max-eigen seeding */
  float early_stop_thresh; /* -early_stop_thresh (default 0: never stop early) */
  int early_stop_range;    /* -early_stop_range (default 5) */
} mrg_fista_params;

void mrg_fista_params_default(mrg_fista_params *p);

/* X (nframes images, overwritten), resid (host, may be NULL): sum|E^H W(Ex-d)|^2 per
 * iteration run, step (host, may be NULL): the 1/max-eigenvalue step size.  With
 * early_stop_thresh > 0 the loop ends once the standard deviation of the last
 * early_stop_range ratios sum|R|^2 / (iteration 0's sum|R|^2) is below it
 * (src/recon_lib.cpp:2081-2087, :2154-2163); mrg_last_iterations gives the count run. */
mrg_status mrg_fista(mrg_plan *plan, const mrg_fista_params *params, void *X, double *resid, float *step,
                     int use_graph, void *stream);

/* CLEAR: per-coil images with a coil low-rank constraint (the CLEAR recon_type,
 * src/recon_lib.cpp:1025-1238; LOWRANKCOIL with dim = 2, src/clear.cpp:99-232, :561-914).
 * Each iteration: R_c = E_c^H W (E_c X_c - d_c) per coil image (E_c without coil maps),
 * step X_c -= (sum |R|^2 / sum P conj(R)) R_c with P_c = E_c^H W E_c R_c, then the coil
 * low-rank threshold of the X_c.  The coil images are combined at the end by the first
 * right singular vector of each block.  Coil maps are not used; frame trajectories and
 * data must be set.  With use_threshold the loop's L1_threshold (src/recon_lib.cpp:
 * 1152-1159, :2416-2527) runs on frame 0's coil images first: wavelet, fraction threshold,
 * soft threshold, with cycle spinning.  ncoil <= 32. */
typedef struct mrg_clear_params {
  int max_iter;            /* -max_iter */
  int block[3];            /* -clear_nx/ny/nz (default 4) */
  int block_iter;          /* -clear_block_iter (default 4) */
  float alpha_coil;        /* -clear_alpha_coil (default 0.01; 0: no threshold) */
  float clear_amp;         /* -clear_amp (default 4) */
  float clear_t2;          /* -clear_t2 (default 6) */
  float early_stop_thresh; /* -early_stop_thresh (default 0: never) */
  int early_stop_range;    /* -early_stop_range (default 5) */
  int64_t rand_skip;       /* rand() draws consumed before the first shift (default 0) */
  int use_threshold;       /* -threshold_type fraction (1) or none (0, default) */
  float thresh;            /* -thresh: fraction of coefficients set to zero */
  int cycle_spins;         /* -cycle_spins (default 4) */
  int wave_levels[3];      /* -wavelet_levelsX/Y/Z (default 4) */
  int wave_type;           /* 0 DB2, 1 DB4 (default) */
} mrg_clear_params;

void mrg_clear_params_default(mrg_clear_params *p);

/* X: nframes combined images (output, host or device).  coil_images (may be NULL): the
 * final per-coil images as nframes x nvox x ncoil complex64, coil innermost (the
 * reference writes them to ClearRaw.h5).  resid (host, may be NULL): sum |R|^2 of each
 * iteration run.  iters (host, may be NULL): iterations run (fewer than max_iter after an
 * early stop). */
mrg_status mrg_clear(mrg_plan *plan, const mrg_clear_params *params, void *X, void *coil_images, double *resid,
                     int *iters, void *stream);

/* Building blocks exposed for drop-in use and parity tests. */
/* LOWRANKCOIL::update_threshold with dim = 2 (src/clear.cpp:99-232) on nframes x nvox x
 * ncoil complex64 (coil innermost): median of the blocks' non-zero sigma_1 times
 * (1 + clear_amp exp(-iteration / clear_t2)) into *smax (host). */
mrg_status mrg_clear_update_threshold(const void *X, int nframes, int ncoil, int Nx, int Ny, int Nz,
                                      const int block[3], float clear_amp, float clear_t2, int iteration,
                                      float *smax, void *stream);
/* LOWRANKCOIL::thresh with dim = 2 (src/clear.cpp:561-813), in place, block shifts drawn
 * from the rand() stream after rand_skip draws. */
mrg_status mrg_clear_thresh(void *X, int nframes, int ncoil, int Nx, int Ny, int Nz, const int block[3],
                            int block_iter, float alpha, float smax, int64_t rand_skip, void *stream);
/* LOWRANKCOIL::combine (src/clear.cpp:815-914): out (nframes x nvox) = A v1 per block,
 * v1 scaled so that its largest-magnitude component is real and positive (a singular
 * vector is defined up to a unit phase); voxels outside whole blocks are left as they are. */
mrg_status mrg_clear_combine(const void *X, int nframes, int ncoil, int Nx, int Ny, int Nz, const int block[3],
                             void *out, void *stream);
/* WAVELET3D::forward/backward (src/wavelet3D.cpp:563-624) on nvol volumes of
 * Nx*Ny*Nz complex64, in place, circular shifts shift[3] (wavelet3D.cpp:443-448). */
mrg_status mrg_wavelet(void *X, int nvol, int Nx, int Ny, int Nz, const int levels[3], const int shift[3],
                       int wave_type, int inverse, void *stream);
/* THRESHOLD::get_threshold for fraction thresholding (src/threshold.cpp:251-391) over
 * nvol volumes of nvox complex64; result written to *value (host). */
mrg_status mrg_fraction_threshold(const void *X, int nvol, int64_t nvox, float fraction, float *value, void *stream);
/* THRESHOLD::thresholding, soft, grouped complex (src/threshold.cpp:766-814). */
mrg_status mrg_soft_threshold(void *X, int64_t n, float value, void *stream);
/* LOWRANKCOIL::update_threshold (src/clear.cpp:233-351) in time, Ne = 1: returns smax. */
mrg_status mrg_llr_update_threshold(const void *X, int nframes, int Nx, int Ny, int Nz, const int block[3],
                                    float clear_amp, float clear_t2, int iteration, float *smax, void *stream);
/* Variant of mrg_llr_update_threshold that allocates no device memory; it has no
 * counterpart in the reference.  For callers that cannot call cudaMalloc (a fixed GPU
 * memory budget reserved up front, or a pipeline that must not synchronise the device
 * between kernels), its scratch lives in a fixed device array of the library, sized for
 * at most MRG_NOALLOC_MAX_BLOCKS low-rank blocks (512 KiB held by every GPU that loads the
 * library until exit); more blocks return MRG_ERR_UNSUPPORTED.  X must be device memory;
 * smax may be host or device memory (a host smax makes the call wait for the result, so
 * inside a stream capture smax must be device memory; a host smax there returns
 * MRG_ERR_INVALID).  The first call on a device looks up the array's device address; make that first call
 * before any stream capture.  All calls share the one array, so calls that overlap on the
 * GPU (other streams or threads) race; serialise them. */
#define MRG_NOALLOC_MAX_BLOCKS 32768
mrg_status mrg_llr_update_threshold_noalloc(const void *X, int nframes, int Nx, int Ny, int Nz, const int block[3],
                                            float clear_amp, float clear_t2, int iteration, float *smax,
                                            void *stream);

/* LOWRANKCOIL::thresh (src/clear.cpp:356-556) in time, Ne = 1, with the block shifts
 * drawn from the rand() stream after rand_skip draws. */
mrg_status mrg_llr_thresh(void *X, int nframes, int Nx, int Ny, int Nz, const int block[3], int block_iter,
                          float alpha, float smax, int64_t rand_skip, void *stream);

/* gaussian_blur (src/ArrayTemplates.cpp:489-601) of nvol complex64 volumes in place
 * (volume c at X + c*vol_stride), sigma per axis (x, y, z; <= 0 skips the axis).  Taps
 * ii in [max(i - w, 0), min(i + w, n)) with w = (int)(5 sigma), as the reference's loop. */
mrg_status mrg_gaussian_blur(void *X, int nvol, int Nx, int Ny, int Nz, int64_t vol_stride, const float sigma[3],
                             void *stream);
/* RECON::sos_normalize with smap_thresh == 0 (src/recon_lib.cpp:3043-3062): each coil
 * divided by sqrt(sum_c |map_c|^2), coil c at maps + c*coil_stride, nvox voxels. */
mrg_status mrg_sos_normalize(void *maps, int ncoil, int64_t coil_stride, int64_t nvox, void *stream);

/* Pipe density compensation, RECON::dcf_calc (src/recon_lib.cpp:854-917) with the
 * DCFgridFFT gridder (src/DCFgridFFT.cpp): kw (M floats, written) from the trajectory
 * of one encode by `iters` rounds of Kw <- Kw / (G^T G Kw) with the polynomial kernel on
 * a (int)(overgrid*N + 16)^3 real grid, then the |k|-dependent width correction and |Kw|.
 * Nx, Ny, Nz: the reconstruction matrix (rcxres, rcyres, rczres).  params may be NULL
 * (the reference's defaults: -dcf_iter 20, -dcf_dwin 2.1, -dcf_scale 1, -dcf_overgrid
 * 2.1, -dcf_acc 1, POLY_KERNEL). */
typedef struct mrg_dcf_params {
  int iters;       /* -dcf_iter */
  float dwin;      /* -dcf_dwin: kernel half width in grid points */
  float scale;     /* -dcf_scale: trajectory scale during the estimate */
  float overgrid;  /* -dcf_overgrid */
  float acc;       /* -dcf_acc: kernel widening with |k| */
  int kernel;      /* 0 POLY_KERNEL, 1 POLY_KERNEL2 (src/DCFgridFFT.h:22-23) */
} mrg_dcf_params;
void mrg_dcf_params_default(mrg_dcf_params *p);
mrg_status mrg_dcf_pipe(const float *kx, const float *ky, const float *kz, int64_t M, int Nx, int Ny, int Nz,
                        const mrg_dcf_params *params, float *kw, void *stream);

/* Host-only (no GPU needed): the geometry and tables mrg_plan_create would build,
 * i.e. gridFFT::precalc_gridding's S, og_s, grid ratio, Kaiser beta and the LUT / window
 * tables (src/gridFFT.cpp:276-643).  lut (3*lut_len) and win (Sx+Sy+Sz) may be NULL
 * to query sizes first. */
mrg_status mrg_plan_geometry(const mrg_config *cfg, int Nx, int Ny, int Nz, int S[3], int og[3], float grid[3],
                             float beta[3], int *lut_len, float *lut, float *win);
/* Gating (host-only, no GPU needed).  Samples are flat in the reference's (readout,
 * projection, slice) order, readout fastest: sample s belongs to readout r = s / nread.
 * gate_times (nreadouts doubles) is GATING::gate_times of one encode (the frame index of
 * each readout as a real number; computing it from ECG / respiratory / time signals is the
 * gating subsystem's job and not done here); rweight (nreadouts floats, may be NULL) the
 * respiratory weight GATING::weight_data multiplies in first (src/gating.cpp:1080-1094).
 * The frame weight of readout r is Tw = rweight[r] * (floor(gate_times[r]) == frame),
 * GATING::hist_weight (src/gating.cpp:1130-1139).
 *   mrg_gate_weights: kw_out[s] = kw[s] * Tw(r) -- the time weight the loops apply when the
 *     data are not pregated (src/recon_lib.cpp:1543-1557); kw_out may alias kw.
 *   mrg_pregate: RECON::pregate_data (src/recon_lib.cpp:675-776) for one frame: the samples
 *     with Tw > 0, in order, into kx/ky/kz/kw_out, kw scaled by 1e6 / count (in the
 *     reference's float / double mix), or 1 with reset_dens, and the ncoil data arrays
 *     (coil c at data + c*coil_stride into data_out + c*out_stride, complex64; both may be
 *     NULL).  *count receives the frame's sample count; with every output NULL only the
 *     count is computed, to size the outputs. */
mrg_status mrg_gate_weights(const double *gate_times, const float *rweight, int64_t nreadouts, int nread, int frame,
                            const float *kw, float *kw_out);
mrg_status mrg_pregate(const double *gate_times, const float *rweight, int64_t nreadouts, int nread, int frame,
                       int reset_dens, const float *kx, const float *ky, const float *kz, const float *kw,
                       const void *data, int ncoil, int64_t coil_stride, float *kx_out, float *ky_out, float *kz_out,
                       float *kw_out, void *data_out, int64_t out_stride, int64_t *count);

/* Reader of the reference's k-space files (MRI_DATA::read_external_data,
 * src/mri_data.cpp:769-906) without the HDF5 library: the subset of the HDF5 format they use
 * (superblocks 0-3, symbol-table and compact link groups, object headers 1 and 2,
 * contiguous and compact datasets of little-endian integers, IEEE floats and (real, imag)
 * float compounds, scalar attributes).  Chunked / compressed datasets and dense groups
 * return MRG_ERR_UNSUPPORTED; a damaged file (truncated, corrupted sizes or addresses)
 * returns MRG_ERR_INVALID, and no read or allocation goes beyond what the file can hold.
 * Host-only except mrg_h5_load_encode.
 *   mrg_h5_attr_int: an integer attribute of a group ("Kdata", "Num_Coils");
 *   mrg_h5_dataset_info: rank and dimensions (HDF5 order: the slowest first) of a dataset;
 *   mrg_h5_read: a whole dataset converted to float32 (complex_out = 0) or complex64, n
 *     elements, into a host buffer;
 *   mrg_h5_mri_info: Num_Encodings, Num_Coils and the samples per encode (size of KX_E<e>,
 *     up to max_encodings of them);
 *   mrg_h5_load_encode: KX/KY/KZ/KW_E<e> and KData_E<e>_C<c> of one encode read into pinned
 *     host memory and set as a plan frame's trajectory and data (mrg_set_traj, mrg_set_data). */
typedef struct mrg_h5 mrg_h5;
mrg_status mrg_h5_open(const char *path, mrg_h5 **out);
mrg_status mrg_h5_close(mrg_h5 *h);
mrg_status mrg_h5_attr_int(mrg_h5 *h, const char *group, const char *name, int *value);
mrg_status mrg_h5_dataset_info(mrg_h5 *h, const char *path, int *rank, int64_t dims[8], int *is_complex);
mrg_status mrg_h5_read(mrg_h5 *h, const char *path, int complex_out, void *dst, int64_t n);
mrg_status mrg_h5_mri_info(mrg_h5 *h, int *num_encodings, int *num_coils, int64_t *samples, int max_encodings);
mrg_status mrg_h5_load_encode(mrg_h5 *h, int encode, mrg_plan *plan, int frame, void *stream);

/* Host-only: n values of the glibc rand() stream for the default seed after `skip`
 * draws, the source of the reference's wavelet and block shifts
 * (src/wavelet3D.cpp:443-448, src/clear.cpp:408-410). */
mrg_status mrg_rand_stream(int64_t skip, int n, int *out);

/* Per-stage device timing, the -time_grid stages of src/gridFFT.cpp:727-778 split at
 * this build's kernels.  While enabled, operator calls run eagerly (no graph), each
 * stage is bracketed by CUDA events and its time accumulated:
 *   out[0..3] E:   set_image+x FFT, z FFT, y FFT, ungrid (chop_grid_backward)
 *   out[4..7] E^H: grid (chop_grid_forward), y FFT, z FFT, x FFT+accumulate
 * (single-coil plans run the FFT axes in the reference's order: z, y, x for E, x, y, z for E^H).
 * mrg_last_timings returns the accumulated ms and the number of operator calls
 * since the previous read, then resets them. */
mrg_status mrg_set_timing(mrg_plan *plan, int enable);
mrg_status mrg_last_timings(mrg_plan *plan, float out[8], int *calls);

/* Number of kernels this library launched since load (process-wide counter). */
int64_t mrg_kernel_launches(void);

/* Bounded device-side waits (no counterpart in the reference, whose loops run on the
 * host).  The tensor-core gridding kernel synchronises its warps through shared-memory
 * barriers; every such wait gives up after `seconds` of GPU time (default 2), records
 * the failure in the plan and returns, leaving the context usable.  A call that waits for
 * the GPU before it returns (host buffers, mrg_cg, mrg_fista, mrg_clear, mrg_grad,
 * mrg_cg_residuals) then returns MRG_ERR_TIMEOUT; calls that return without waiting
 * (device buffers, mrg_cg_iterate) leave it to the next waiting call or to
 * mrg_plan_check.  The record is cleared when it is reported.  0 makes a wait give up
 * after its first unsuccessful try (for tests). */
mrg_status mrg_set_wait_limit(mrg_plan *plan, double seconds);
/* Waits for `stream` and reports (MRG_ERR_TIMEOUT) and clears a wait that ran out in this
 * plan's kernels since the last report. */
mrg_status mrg_plan_check(mrg_plan *plan, void *stream);
/* Iterations the last mrg_cg / mrg_fista / mrg_clear on this plan ran (fewer than max_iter
 * after an early stop). */
mrg_status mrg_last_iterations(const mrg_plan *plan, int *iters);

#ifdef __cplusplus
}
#endif

#endif /* MRG_H */
