// C entry points over the reference's own gridFFT, gridFFT_CoilThreaded, DCFgridFFT,
// WAVELET3D, THRESHOLD, LOWRANKCOIL and SPIRIT classes (src/gridFFT.cpp,
// src/gridFFT_CoilThreaded.cpp, src/DCFgridFFT.cpp, src/ArrayTemplates.cpp,
// src/wavelet3D.cpp, src/threshold.cpp, src/clear.cpp, src/spirit.cpp compiled unmodified
// against the stand-in headers in refshim/), for checking the oracle
// restatement against the reference itself.  Test infrastructure only: built into
// oracle/_ref/libref.so by `make -C oracle ref` where the reference sources are present,
// and loaded only by tests/test_oracle_ref.py.
//
// Layouts: images are C-order (Nz, Ny, Nx) complex64, i.e. x fastest, which is the
// memory order of the reference's column-major Blitz arrays (Nx, Ny, Nz); k-space and
// trajectories are flat arrays of M samples, an (M, 1, 1) column-major array; the
// oversampled grid is (Sz, Sy, Sx).
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "DCFgridFFT.h"
#include "clear.h"
#include "gridFFT.h"
#include "gridFFT_CoilThreaded.h"
#include "spirit.h"
#include "threshold.h"
#include "wavelet3D.h"

using namespace NDarray;
typedef std::complex<float> cf;

// MRI_DATA's constructor lives in src/mri_data.cpp, which needs HDF5 and Armadillo; the
// gridding set-up reads only trajectory_type and dft_needed, which the driver sets.
MRI_DATA::MRI_DATA(void) {}

namespace {

template <typename T>
Array<T, 3> col3(int n0, int n1, int n2, const void *src) {
  Array<T, 3> a;
  a.setStorage(ColumnMajorArray<3>());
  a.resize(n0, n1, n2);
  if (src) std::memcpy(a.data(), src, sizeof(T) * (size_t)n0 * n1 * n2);
  else a = T(0);
  return a;
}

struct Config {
  float overgrid, dwin;
  int kernel_type;
  float k_rad;
};

// gridFFT set up as the reference's callers do: public fields first, then
// precalc_gridding(Nz, Ny, Nx, data) for a 3D non-Cartesian acquisition.
void setup(gridFFT &g, const Config &c, int Nx, int Ny, int Nz) {
  g.overgrid = c.overgrid;
  g.kernel_type = c.kernel_type;
  if (c.dwin > 0.0f) g.dwinX = g.dwinY = g.dwinZ = c.dwin;
  g.k_rad = c.k_rad;
  MRI_DATA data;
  for (int d = 0; d < 3; d++) {
    data.trajectory_type(d) = MRI_DATA::NONCARTESIAN;
    data.dft_needed(d) = true;
  }
  data.Num_Coils = 1;
  g.precalc_gridding(Nz, Ny, Nx, data);
}

// LOWRANKCOIL as recon_lib's loops use it, with the block edges update_threshold leaves
// in its members (clamped to the image) and the rand() stream of a process that seeded it
// with srand(1) and has drawn `skip` numbers since.
LOWRANKCOIL lowrank(const int *bs, int Nx, int Ny, int Nz, int block_iter, float amp, float t2) {
  LOWRANKCOIL lr;
  lr.block_size_x = std::min(bs[0], Nx);
  lr.block_size_y = std::min(bs[1], Ny);
  lr.block_size_z = std::min(bs[2], Nz);
  lr.block_iter = block_iter;
  lr.clear_amp = amp;
  lr.clear_t2 = t2;
  return lr;
}

void seed_rand(long skip) {
  std::srand(1);
  for (long i = 0; i < skip; i++) std::rand();
}

// Nt frames (Ne = 1) of one image each, vols[t] -> image(t, 0)
Array<Array<cf, 3>, 2> frames(void **vols, int Nt, int Nx, int Ny, int Nz) {
  Array<Array<cf, 3>, 2> im;
  im.setStorage(ColumnMajorArray<2>());
  im.resize(Nt, 1);
  for (int t = 0; t < Nt; t++) im(t, 0).reference(col3<cf>(Nx, Ny, Nz, vols[t]));
  return im;
}

// Nt frames (Ne = 1) of C coil images, vols[t * C + c] -> image(t, 0, c)
Array<Array<cf, 3>, 3> coil_frames(void **vols, int Nt, int C, int Nx, int Ny, int Nz) {
  Array<Array<cf, 3>, 3> im;
  im.setStorage(ColumnMajorArray<3>());
  im.resize(Nt, 1, C);
  for (int t = 0; t < Nt; t++)
    for (int c = 0; c < C; c++) im(t, 0, c).reference(col3<cf>(Nx, Ny, Nz, vols[t * C + c]));
  return im;
}

// gridFFT_CoilThreaded set up the same way, with the coil count in MRI_DATA
// (precalc_gridding allocates one grid per coil from it)
void setup_coils(gridFFT_CoilThreaded &g, const Config &c, int Nx, int Ny, int Nz, int C) {
  g.overgrid = c.overgrid;
  g.kernel_type = c.kernel_type;
  if (c.dwin > 0.0f) g.dwinX = g.dwinY = g.dwinZ = c.dwin;
  g.k_rad = c.k_rad;
  MRI_DATA data;
  for (int d = 0; d < 3; d++) {
    data.trajectory_type(d) = MRI_DATA::NONCARTESIAN;
    data.dft_needed(d) = true;
  }
  data.Num_Coils = C;
  g.precalc_gridding(Nz, Ny, Nx, data);
}

// C arrays of n0 x n1 x n2 (column-major) over the caller's buffers, copied in
Complex4D coil_arrays(void *const *bufs, int C, int n0, int n1, int n2) {
  Complex4D a(C);
  for (int c = 0; c < C; c++) a(c).reference(col3<cf>(n0, n1, n2, bufs ? bufs[c] : nullptr));
  return a;
}

struct Traj {
  Array<float, 3> kx, ky, kz, kw;
  Traj(const float *x, const float *y, const float *z, const float *w, long M)
      : kx(col3<float>((int)M, 1, 1, x)), ky(col3<float>((int)M, 1, 1, y)), kz(col3<float>((int)M, 1, 1, z)),
        kw(col3<float>((int)M, 1, 1, w)) {}
};

// S, og_s, beta, kernel tables and windows of a gridder after precalc_gridding
template <class G>
int copy_tables(const G &g, int *S, int *og, float *beta, int *lut_len, float *lut, float *win) {
  S[0] = g.Sx, S[1] = g.Sy, S[2] = g.Sz;
  og[0] = g.og_sx, og[1] = g.og_sy, og[2] = g.og_sz;
  beta[0] = g.betaX, beta[1] = g.betaY, beta[2] = g.betaZ;
  const Array<float, 1> *f[3] = {&g.grid_filterX, &g.grid_filterY, &g.grid_filterZ};
  *lut_len = (int)f[0]->numElements();
  if (lut)
    for (int d = 0; d < 3; d++) {
      if (f[d]->numElements() != *lut_len) return 1;
      for (int i = 0; i < *lut_len; i++) lut[d * *lut_len + i] = (*f[d])(i);
    }
  if (win) {
    int o = 0;
    for (int i = 0; i < g.Sx; i++) win[o++] = g.winx(i);
    for (int i = 0; i < g.Sy; i++) win[o++] = g.winy(i);
    for (int i = 0; i < g.Sz; i++) win[o++] = g.winz(i);
  }
  return 0;
}

}  // namespace

extern "C" {

// precalc_gridding: S, og_s, beta, the kernel tables grid_filterX/Y/Z (lut_len each, lut may
// be NULL) and the windows winx/winy/winz (Sx + Sy + Sz floats, may be NULL).
int ref_tables(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, int *S, int *og, float *beta,
               int *lut_len, float *lut, float *win) {
  gridFFT g;
  setup(g, Config{overgrid, dwin, kernel_type, 9999.0f}, Nx, Ny, Nz);
  return copy_tables(g, S, og, beta, lut_len, lut, win);
}

// The same from gridFFT_CoilThreaded::precalc_gridding (src/gridFFT_CoilThreaded.cpp:403-568)
// for C coils.
int ref_coils_tables(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, int C, int *S, int *og,
                     float *beta, int *lut_len, float *lut, float *win) {
  gridFFT_CoilThreaded g;
  setup_coils(g, Config{overgrid, dwin, kernel_type, 9999.0f}, Nx, Ny, Nz, C);
  return copy_tables(g, S, og, beta, lut_len, lut, win);
}

// gridFFT::backward (E) or backward_residual (diff != NULL): data = E(X smap) (- diff).
int ref_forward(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, float k_rad, const void *X,
                const void *smap, const float *kx, const float *ky, const float *kz, const float *kw, long M,
                void *data, const void *diff) {
  gridFFT g;
  setup(g, Config{overgrid, dwin, kernel_type, k_rad}, Nx, Ny, Nz);
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, X), s = col3<cf>(Nx, Ny, Nz, smap), d = col3<cf>((int)M, 1, 1, nullptr);
  Traj t(kx, ky, kz, kw, M);
  if (diff) {
    Array<cf, 3> df = col3<cf>((int)M, 1, 1, diff);
    g.backward_residual(x, s, d, t.kx, t.ky, t.kz, t.kw, df);
  } else {
    g.backward(x, s, d, t.kx, t.ky, t.kz, t.kw);
  }
  std::memcpy(data, d.data(), sizeof(cf) * (size_t)M);
  return 0;
}

// gridFFT::forward (E^H) with a map: X += E^H(data) conj(smap), X read and written.
int ref_adjoint(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, float k_rad, void *X,
                const void *smap, const void *data, const float *kx, const float *ky, const float *kz, const float *kw,
                long M) {
  gridFFT g;
  setup(g, Config{overgrid, dwin, kernel_type, k_rad}, Nx, Ny, Nz);
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, X), s = col3<cf>(Nx, Ny, Nz, smap), d = col3<cf>((int)M, 1, 1, data);
  Traj t(kx, ky, kz, kw, M);
  g.forward(x, s, d, t.kx, t.ky, t.kz, t.kw);
  std::memcpy(X, x.data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// chop_grid_forward into a zeroed grid (Sz, Sy, Sx), written to `grid`.
int ref_grid(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, float k_rad, const void *data,
             const float *kx, const float *ky, const float *kz, const float *kw, long M, void *grid) {
  gridFFT g;
  setup(g, Config{overgrid, dwin, kernel_type, k_rad}, Nx, Ny, Nz);
  Array<cf, 3> d = col3<cf>((int)M, 1, 1, data);
  Traj t(kx, ky, kz, kw, M);
  g.k3d_grid = cf(0.0f, 0.0f);
  g.chop_grid_forward(d, t.kx, t.ky, t.kz, t.kw);
  std::memcpy(grid, g.k3d_grid.data(), sizeof(cf) * (size_t)g.Sx * g.Sy * g.Sz);
  return 0;
}

// chop_grid_backward from a caller grid (Sz, Sy, Sx): data = taps * grid (- diff).
int ref_ungrid(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, const void *grid, const float *kx,
               const float *ky, const float *kz, const float *kw, long M, void *data, const void *diff) {
  gridFFT g;
  setup(g, Config{overgrid, dwin, kernel_type, 9999.0f}, Nx, Ny, Nz);
  std::memcpy(g.k3d_grid.data(), grid, sizeof(cf) * (size_t)g.Sx * g.Sy * g.Sz);
  Array<cf, 3> d = col3<cf>((int)M, 1, 1, nullptr);
  Array<cf, 3> df = diff ? col3<cf>((int)M, 1, 1, diff) : Array<cf, 3>();
  Traj t(kx, ky, kz, kw, M);
  g.chop_grid_backward(d, t.kx, t.ky, t.kz, t.kw, df, diff != nullptr);
  std::memcpy(data, d.data(), sizeof(cf) * (size_t)M);
  return 0;
}

// do_fft (pruned: the input is read inside the crop only) or do_ifft on a caller grid.
int ref_fft(int Nx, int Ny, int Nz, float overgrid, int inverse, void *grid) {
  gridFFT g;
  setup(g, Config{overgrid, -1.0f, KAISER_KERNEL, 9999.0f}, Nx, Ny, Nz);
  const size_t n = (size_t)g.Sx * g.Sy * g.Sz;
  std::memcpy(g.k3d_grid.data(), grid, sizeof(cf) * n);
  if (inverse) g.do_ifft();
  else g.do_fft();
  std::memcpy(grid, g.k3d_grid.data(), sizeof(cf) * n);
  return 0;
}

// gridFFT::forward_sos (src/gridFFT.cpp:722-748): X += |E^H data, deapodised|^2, X read and written.
int ref_adjoint_sos(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, float k_rad, void *X,
                    const void *data, const float *kx, const float *ky, const float *kz, const float *kw, long M) {
  gridFFT g;
  setup(g, Config{overgrid, dwin, kernel_type, k_rad}, Nx, Ny, Nz);
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, X), d = col3<cf>((int)M, 1, 1, data);
  Traj t(kx, ky, kz, kw, M);
  g.forward_sos(x, d, t.kx, t.ky, t.kz, t.kw);
  std::memcpy(X, x.data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// gridFFT_CoilThreaded::backward (E of C coils) or backward_residual (diff != NULL):
// data[c] = E(X smap[c]) (- diff[c]), M samples each.
int ref_coils_forward(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, float k_rad, int C,
                      const void *X, void *const *smaps, const float *kx, const float *ky, const float *kz,
                      const float *kw, long M, void *const *data, void *const *diff) {
  gridFFT_CoilThreaded g;
  setup_coils(g, Config{overgrid, dwin, kernel_type, k_rad}, Nx, Ny, Nz, C);
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, X);
  Complex4D s = coil_arrays(smaps, C, Nx, Ny, Nz), d = coil_arrays(nullptr, C, (int)M, 1, 1);
  Traj t(kx, ky, kz, kw, M);
  if (diff) {
    Complex4D df = coil_arrays(diff, C, (int)M, 1, 1);
    g.backward_residual(x, s, d, t.kx, t.ky, t.kz, t.kw, df);
  } else {
    g.backward(x, s, d, t.kx, t.ky, t.kz, t.kw);
  }
  for (int c = 0; c < C; c++) std::memcpy(data[c], d(c).data(), sizeof(cf) * (size_t)M);
  return 0;
}

// gridFFT_CoilThreaded::forward (E^H of C coils with maps): X += sum_c E^H(data[c]) conj(smap[c]).
int ref_coils_adjoint(int Nx, int Ny, int Nz, float overgrid, float dwin, int kernel_type, float k_rad, int C,
                      void *X, void *const *smaps, void *const *data, const float *kx, const float *ky,
                      const float *kz, const float *kw, long M) {
  gridFFT_CoilThreaded g;
  setup_coils(g, Config{overgrid, dwin, kernel_type, k_rad}, Nx, Ny, Nz, C);
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, X);
  Complex4D s = coil_arrays(smaps, C, Nx, Ny, Nz), d = coil_arrays(data, C, (int)M, 1, 1);
  Traj t(kx, ky, kz, kw, M);
  g.forward(x, s, d, t.kx, t.ky, t.kz, t.kw);
  std::memcpy(X, x.data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// DCFgridFFT::precalc_kernel's table (src/DCFgridFFT.cpp:54-164) for the half width
// dwin and the kernel (0 POLY_KERNEL, 1 POLY_KERNEL2): *len entries into out (NULL: the
// length only).
int ref_dcf_table(float dwin, int kernel, float *out, int *len) {
  DCFgridFFT dcf;
  dcf.kernel_type = kernel;
  dcf.dwinX = dcf.dwinY = dcf.dwinZ = dwin;
  dcf.precalc_kernel();
  *len = (int)dcf.grid_filterX.numElements();
  if (out)
    for (int i = 0; i < *len; i++) out[i] = dcf.grid_filterX(i);
  return 0;
}

// RECON::dcf_calc (src/recon_lib.cpp:855-912, which src/recon_lib.cpp cannot be compiled
// here to provide) for one encode, around the reference's own DCFgridFFT: the gridder set
// up as there, the trajectory scaled by `scale`, `iters` Pipe iterations from kw = 1
// (kw <- kw / (grid then degrid of kw), 0 where that is below 1e-3), then scale_kw and the
// magnitude.  kernel 0 is DCFgridFFT::POLY_KERNEL (recon_lib's choice), 1 POLY_KERNEL2.
int ref_dcf_pipe(const float *kx, const float *ky, const float *kz, long M, int Nx, int Ny, int Nz, int iters,
                 float dwin, float scale, float overgrid, float acc, int kernel, float *kw_out) {
  DCFgridFFT dcf;
  dcf.kernel_type = kernel;
  dcf.dwinX = dcf.dwinY = dcf.dwinZ = dwin;
  dcf.grid_x = dcf.grid_y = dcf.grid_z = overgrid;
  dcf.grid_in_x = dcf.grid_in_y = dcf.grid_in_z = 1;
  dcf.precalc_kernel();
  dcf.acc = acc;
  // the image's extents as the float expressions overgrid * N + 16 converted to int
  Array<float, 3> X((int)(overgrid * Nz + 16), (int)(overgrid * Ny + 16), (int)(overgrid * Nx + 16),
                    ColumnMajorArray<3>());
  Array<float, 3> tx = col3<float>((int)M, 1, 1, kx), ty = col3<float>((int)M, 1, 1, ky),
                  tz = col3<float>((int)M, 1, 1, kz);
  tx *= scale;
  ty *= scale;
  tz *= scale;
  Array<float, 3> w = col3<float>((int)M, 1, 1, nullptr), w2 = col3<float>((int)M, 1, 1, nullptr);
  w = 1;
  for (int it = 0; it < iters; it++) {
    X = 0;
    w2 = 0.0;
    dcf.forward(X, w, tx, ty, tz);
    dcf.backward(X, w2, tx, ty, tz);
    for (long i = 0; i < M; i++) {
      float &a = w(i, 0, 0);
      const float b = w2(i, 0, 0);
      if (std::abs(b) < 1e-3) a = 0.0f;
      else a = a / b;
    }
  }
  dcf.scale_kw(w, tx, ty, tz);
  for (long i = 0; i < M; i++) kw_out[i] = std::abs(w(i, 0, 0));
  return 0;
}

// SPIRIT::generateEigenCoils (src/spirit.cpp:137-172) as recon_lib calls it
// (src/recon_lib.cpp:2895-2898): the kernel radii, calibration radii, singular-value
// threshold and calibration shape set as read_commandline sets them from -sp_krx_f ..
// -sp_square, init with the image size and coil count, then C coil images of one encode
// (transformed in place) -> C maps.
int ref_espirit(void *const *imgs, int C, int Nx, int Ny, int Nz, const float *kr_f, const int *cr,
                float svd_thresh, int square, void *const *maps) {
  SPIRIT sp;
  sp.krx_f = kr_f[0];
  sp.kry_f = kr_f[1];
  sp.krz_f = kr_f[2];
  sp.crx = cr[0];
  sp.cry = cr[1];
  sp.crz = cr[2];
  sp.svd_thresh = svd_thresh;
  sp.shape = square ? SP_SQUARE : SP_CIRCLE;
  sp.init(Nx, Ny, Nz, C);
  Array<Array<cf, 3>, 2> image;
  image.setStorage(ColumnMajorArray<2>());
  image.resize(1, C);
  for (int c = 0; c < C; c++) image(0, c).reference(col3<cf>(Nx, Ny, Nz, imgs[c]));
  Complex4D sm = coil_arrays(nullptr, C, Nx, Ny, Nz);
  sp.generateEigenCoils(sm, image);
  for (int c = 0; c < C; c++) std::memcpy(maps[c], sm(c).data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// NDarray::gaussian_blur (src/ArrayTemplates.cpp:489-608) of one complex volume in place,
// sigma per axis (x, y, z).
int ref_gaussian_blur(void *X, int Nx, int Ny, int Nz, const float *sigma) {
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, X);
  gaussian_blur(x, sigma[0], sigma[1], sigma[2]);
  std::memcpy(X, x.data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// WAVELET3D forward (inverse = 0) or backward of one volume in place, with the shifts S set
// as random_shift would have set them.
int ref_wavelet(int Nx, int Ny, int Nz, const int *levels, const int *shift, int wave_type, int inverse, void *X) {
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, X);
  int l[3] = {levels[0], levels[1], levels[2]};
  WAVELET3D w(x, l, wave_type);
  for (int d = 0; d < 3; d++) w.S[d] = shift[d];
  if (inverse) w.backward(x);
  else w.forward(x);
  std::memcpy(X, x.data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// WAVELET3D::random_shift (src/wavelet3D.cpp:443-448) called n times on a transform of
// the given type and shape, rand() seeded with srand(1) and advanced `skip` draws: the
// shifts (x, y, z) of each call into S (3n ints), as L1_threshold's cycle spins draw them.
int ref_wavelet_shifts(int Nx, int Ny, int Nz, const int *levels, int wave_type, long skip, int n, int *S) {
  Array<cf, 3> x = col3<cf>(Nx, Ny, Nz, nullptr);
  int l[3] = {levels[0], levels[1], levels[2]};
  WAVELET3D w(x, l, wave_type);
  seed_rand(skip);
  for (int i = 0; i < n; i++) {
    w.random_shift();
    for (int d = 0; d < 3; d++) S[3 * i + d] = w.S[d];
  }
  return 0;
}

// THRESHOLD with -threshold_type fraction -thresh <fraction>: update_threshold over nvol
// volumes (frames) gives global_threshold; with apply != 0 exec_threshold then soft
// thresholds the volumes in place.  Returns the threshold.
float ref_fraction_threshold(int Nx, int Ny, int Nz, int nvol, void **vols, float fraction, int apply) {
  char val[64];
  std::snprintf(val, sizeof(val), "%.9g", fraction);
  const char *args[] = {"-threshold_type", "fraction", "-thresh", val};
  THRESHOLD th(4, args);
  th.VERBOSE = false;
  Array<Array<cf, 3>, 2> coef;
  coef.setStorage(ColumnMajorArray<2>());
  coef.resize(nvol, 1);
  for (int t = 0; t < nvol; t++) coef(t, 0).reference(col3<cf>(Nx, Ny, Nz, vols[t]));
  WAVELET3D wave;
  th.update_threshold(coef, wave, 1.0f);
  if (apply) {
    th.exec_threshold(coef, wave);
    for (int t = 0; t < nvol; t++) std::memcpy(vols[t], coef(t, 0).data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  }
  return th.global_threshold;
}

// LOWRANKCOIL::update_threshold(image, 0, iter) over Nt frames: the time low-rank smax.
float ref_llr_update_threshold(void **vols, int Nt, int Nx, int Ny, int Nz, const int *bs, float amp, float t2,
                               int iter) {
  LOWRANKCOIL lr = lowrank(bs, Nx, Ny, Nz, 1, amp, t2);
  Array<Array<cf, 3>, 2> im = frames(vols, Nt, Nx, Ny, Nz);
  lr.update_threshold(im, 0, iter);
  return lr.smax;
}

// LOWRANKCOIL::thresh(image, 0) in place, with clear_alpha_time = alpha and the given smax.
int ref_llr_thresh(void **vols, int Nt, int Nx, int Ny, int Nz, const int *bs, int block_iter, float alpha,
                   float smax, long rand_skip) {
  LOWRANKCOIL lr = lowrank(bs, Nx, Ny, Nz, block_iter, 4.0f, 6.0f);
  lr.clear_alpha_time = alpha;
  lr.smax = smax;
  Array<Array<cf, 3>, 2> im = frames(vols, Nt, Nx, Ny, Nz);
  seed_rand(rand_skip);
  lr.thresh(im, 0);
  for (int t = 0; t < Nt; t++) std::memcpy(vols[t], im(t, 0).data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// LOWRANKCOIL::update_threshold(image, 2, iter) over Nt frames of C coil images.
float ref_clear_update_threshold(void **vols, int Nt, int C, int Nx, int Ny, int Nz, const int *bs, float amp,
                                 float t2, int iter) {
  LOWRANKCOIL lr = lowrank(bs, Nx, Ny, Nz, 1, amp, t2);
  Array<Array<cf, 3>, 3> im = coil_frames(vols, Nt, C, Nx, Ny, Nz);
  lr.update_threshold(im, 2, iter);
  return lr.smax;
}

// LOWRANKCOIL::thresh(image, 2) in place, with clear_alpha_coil = alpha and the given smax.
int ref_clear_thresh(void **vols, int Nt, int C, int Nx, int Ny, int Nz, const int *bs, int block_iter, float alpha,
                     float smax, long rand_skip) {
  LOWRANKCOIL lr = lowrank(bs, Nx, Ny, Nz, block_iter, 4.0f, 6.0f);
  lr.clear_alpha_coil = alpha;
  lr.smax = smax;
  Array<Array<cf, 3>, 3> im = coil_frames(vols, Nt, C, Nx, Ny, Nz);
  seed_rand(rand_skip);
  lr.thresh(im, 2);
  for (int t = 0; t < Nt; t++)
    for (int c = 0; c < C; c++)
      std::memcpy(vols[t * C + c], im(t, 0, c).data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

// LOWRANKCOIL::combine(image, out): out[t] (Nt images, updated where blocks cover them).
int ref_clear_combine(void **vols, int Nt, int C, int Nx, int Ny, int Nz, const int *bs, void **out) {
  LOWRANKCOIL lr = lowrank(bs, Nx, Ny, Nz, 1, 4.0f, 6.0f);
  Array<Array<cf, 3>, 3> im = coil_frames(vols, Nt, C, Nx, Ny, Nz);
  Array<Array<cf, 3>, 2> o = frames(out, Nt, Nx, Ny, Nz);
  lr.combine(im, o);
  for (int t = 0; t < Nt; t++) std::memcpy(out[t], o(t, 0).data(), sizeof(cf) * (size_t)Nx * Ny * Nz);
  return 0;
}

}  // extern "C"
