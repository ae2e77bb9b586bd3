// gridfft_gb300.hpp -- header-only C++ drop-in for uwmri/mri_recon's gridFFT and
// gridFFT_CoilThreaded (src/gridFFT.h:28-194, src/gridFFT_CoilThreaded.h:26-191)
// over the C ABI of mrg.h.
//
// The member functions keep the reference's names and argument meaning; Blitz
// arrays become raw pointers plus a sample count:
//   forward(X, smap, data, kx, ky, kz, kw, M)            X += E^H (data * kw)
//   backward(X, smap, data, kx, ky, kz, kw, M)           data = E X
//   backward_residual(X, smap, data, kx, ky, kz, kw, M, diff)   data = E X - diff
//   forward_sos(X, data, kx, ky, kz, kw, M)              X += |deapp(E^H (data * kw))|^2
// Images are complex<float>[Nz][Ny][Nx] (x fastest), k-space complex<float>[M],
// trajectories float[M] in the reference's units.  Pointers may be host or
// device memory.  Errors throw std::runtime_error with the library's message
// instead of exit(1).
// k_rad may be changed between calls, as recon_lib does around the coil-map
// estimate (src/recon_lib.cpp:2738, :2786); the next call applies it.
//
// A trajectory is uploaded and sorted on the first call that passes it and
// reused while the same arrays (same addresses and length) are passed, which is
// how recon_lib's loops use it; call reset_trajectory() after changing the
// contents of an array in place.
#ifndef GRIDFFT_GB300_HPP
#define GRIDFFT_GB300_HPP

#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "mrg.h"

namespace mrg_cxx {

enum { TRIANGLE_KERNEL = MRG_KERNEL_TRIANGLE, KAISER_KERNEL = MRG_KERNEL_KAISER, SINC_KERNEL = MRG_KERNEL_SINC,
       POLY_KERNEL = MRG_KERNEL_POLY };

inline void check(mrg_status s) {
  if (s != MRG_OK) throw std::runtime_error(std::string("mrg: ") + mrg_last_error());
}

typedef std::complex<float> cf;

class gridFFT {
 public:
  // Fields set before precalc_gridding (src/gridFFT.cpp:28-60 defaults).
  float overgrid = 1.5f;
  int kernel_type = KAISER_KERNEL;
  float dwinX = -1.0f, dwinY = -1.0f, dwinZ = -1.0f;
  float k_rad = 9999.0f;
  int time_grid = 0;
  // Filled by precalc_gridding (src/gridFFT.cpp:475-643).
  int Nx = 0, Ny = 0, Nz = 0, Sx = 0, Sy = 0, Sz = 0;
  int og_sx = 0, og_sy = 0, og_sz = 0, og_ex = 0, og_ey = 0, og_ez = 0;
  float grid_x = 0, grid_y = 0, grid_z = 0, betaX = 0, betaY = 0, betaZ = 0;

  gridFFT() = default;
  gridFFT(const gridFFT &) = delete;
  gridFFT &operator=(const gridFFT &) = delete;
  virtual ~gridFFT() {
    if (plan_) mrg_plan_destroy(plan_);
  }

  void precalc_gridding(int NzT, int NyT, int NxT) { setup(NzT, NyT, NxT, 1); }

  void forward(cf *X, const cf *smap, const cf *data, const float *kx, const float *ky, const float *kz,
               const float *kw, int64_t M, void *stream = nullptr) {
    traj(kx, ky, kz, kw, M, stream);
    sync_k_rad(stream);
    check(mrg_adjoint_coil(plan_, 0, smap, data, X, stream));
  }
  void forward_sos(cf *X, const cf *data, const float *kx, const float *ky, const float *kz, const float *kw,
                   int64_t M, void *stream = nullptr) {
    traj(kx, ky, kz, kw, M, stream);
    sync_k_rad(stream);
    check(mrg_adjoint_sos(plan_, 0, data, M, X, stream));
  }
  void backward(const cf *X, const cf *smap, cf *data, const float *kx, const float *ky, const float *kz,
                const float *kw, int64_t M, void *stream = nullptr) {
    traj(kx, ky, kz, kw, M, stream);
    check(mrg_forward_coil(plan_, 0, X, smap, data, nullptr, stream));
  }
  void backward_residual(const cf *X, const cf *smap, cf *data, const float *kx, const float *ky, const float *kz,
                         const float *kw, int64_t M, const cf *diff, void *stream = nullptr) {
    traj(kx, ky, kz, kw, M, stream);
    check(mrg_forward_coil(plan_, 0, X, smap, data, diff, stream));
  }
  void reset_trajectory() { keyM_ = -1; }
  mrg_plan *plan() const { return plan_; }

 protected:
  void setup(int NzT, int NyT, int NxT, int ncoil) {
    if (!(dwinX == dwinY && dwinY == dwinZ)) throw std::runtime_error("mrg: anisotropic kernel widths");
    mrg_config cfg;
    mrg_config_default(&cfg);
    cfg.overgrid = overgrid;
    cfg.dwin = dwinX;
    cfg.kernel_type = kernel_type;
    cfg.k_rad = k_rad;
    cfg.time_grid = time_grid;
    cfg.fft_norm = fft_norm_;
    if (plan_) mrg_plan_destroy(plan_);
    plan_ = nullptr;
    check(mrg_plan_create(&cfg, NxT, NyT, NzT, ncoil, 1, &plan_));
    int S[3], og[3], ll;
    float gr[3], be[3], dw[3];
    check(mrg_plan_info(plan_, S, og, gr, be, dw, &ll));
    Nx = NxT; Ny = NyT; Nz = NzT;
    Sx = S[0]; Sy = S[1]; Sz = S[2];
    og_sx = og[0]; og_sy = og[1]; og_sz = og[2];
    og_ex = og_sx + Nx; og_ey = og_sy + Ny; og_ez = og_sz + Nz;
    grid_x = gr[0]; grid_y = gr[1]; grid_z = gr[2];
    betaX = be[0]; betaY = be[1]; betaZ = be[2];
    dwinX = dw[0]; dwinY = dw[1]; dwinZ = dw[2];
    keyM_ = -1;
    k_rad_set_ = k_rad;
  }
  void sync_k_rad(void *stream) {
    if (k_rad == k_rad_set_) return;
    check(mrg_set_k_rad(plan_, k_rad, stream));
    k_rad_set_ = k_rad;
  }
  void traj(const float *kx, const float *ky, const float *kz, const float *kw, int64_t M, void *stream) {
    if (!plan_) throw std::runtime_error("mrg: precalc_gridding not called");
    if (keyM_ == M && key_[0] == kx && key_[1] == ky && key_[2] == kz && key_[3] == kw) return;
    check(mrg_set_traj(plan_, 0, kx, ky, kz, kw, M, stream));
    key_[0] = kx; key_[1] = ky; key_[2] = kz; key_[3] = kw;
    keyM_ = M;
  }
  mrg_plan *plan_ = nullptr;
  int fft_norm_ = 0;  // mrg_config.fft_norm: 1 for the coil-threaded class's unnormalised FFTs
  const void *key_[4] = {nullptr, nullptr, nullptr, nullptr};
  int64_t keyM_ = -1;
  float k_rad_set_ = 9999.0f;
};

// All coils in one call (the reference's -parallel_coils path).  smaps and data are
// coil-major: coil c at smaps + c*Nx*Ny*Nz and data + c*M.  As the reference's class, it
// defaults to overgrid 1.375 (src/gridFFT_CoilThreaded.cpp:31) and transforms without the
// 1/sqrt(S) per axis of gridFFT (its FFTW calls are unnormalised,
// src/gridFFT_CoilThreaded.cpp:570-893), so its E and E^H are sqrt(Sx Sy Sz) times gridFFT's.
class gridFFT_CoilThreaded : public gridFFT {
 public:
  gridFFT_CoilThreaded() {
    overgrid = 1.375f;
    fft_norm_ = 1;
  }
  void precalc_gridding(int NzT, int NyT, int NxT, int ncoils) {
    setup(NzT, NyT, NxT, ncoils);
    ncoils_ = ncoils;
    smaps_ = nullptr;
  }
  void forward(cf *X, const cf *smaps, const cf *data, const float *kx, const float *ky, const float *kz,
               const float *kw, int64_t M, void *stream = nullptr) {
    traj(kx, ky, kz, kw, M, stream);
    maps(smaps, stream);
    sync_k_rad(stream);
    check(mrg_adjoint(plan_, 0, data, M, X, stream));
  }
  void backward(const cf *X, const cf *smaps, cf *data, const float *kx, const float *ky, const float *kz,
                const float *kw, int64_t M, void *stream = nullptr) {
    traj(kx, ky, kz, kw, M, stream);
    maps(smaps, stream);
    check(mrg_forward(plan_, 0, X, data, M, nullptr, stream));
  }
  void backward_residual(const cf *X, const cf *smaps, cf *data, const float *kx, const float *ky, const float *kz,
                         const float *kw, int64_t M, const cf *diff, void *stream = nullptr) {
    traj(kx, ky, kz, kw, M, stream);
    maps(smaps, stream);
    check(mrg_forward(plan_, 0, X, data, M, diff, stream));
  }
  void reset_maps() { smaps_ = nullptr; }

 private:
  void maps(const cf *smaps, void *stream) {
    if (smaps == smaps_) return;
    check(mrg_set_smaps(plan_, smaps, (int64_t)Nx * Ny * Nz, stream));
    smaps_ = smaps;
  }
  int ncoils_ = 1;
  const cf *smaps_ = nullptr;
};

}  // namespace mrg_cxx

#endif  // GRIDFFT_GB300_HPP
