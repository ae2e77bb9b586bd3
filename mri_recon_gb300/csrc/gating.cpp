// Frame weights and per-frame compaction of gated acquisitions (host code, no GPU):
// GATING::hist_weight (src/gating.cpp:1130-1139), the respiratory factor of
// GATING::weight_data (src/gating.cpp:1080-1094) and RECON::pregate_data
// (src/recon_lib.cpp:675-776).  Samples are flat in the reference's (readout, projection,
// slice) column-major order, readout fastest, so sample s belongs to readout r = s / nread,
// the (projection, slice) element of the per-readout gate times and weights.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "mrg_internal.h"

using namespace mrg;

namespace {

bool gate_args_ok(const double *gate_times, int64_t nreadouts, int nread) {
  if (!gate_times || nreadouts < 0 || nread < 1 || nreadouts > INT64_MAX / nread) {
    set_error("bad gating arguments");
    return false;
  }
  return true;
}

// Tw of readout r for frame t: rweight[r] (1 when absent) times the hist mask
inline float frame_weight(const double *gate_times, const float *rweight, int64_t r, int t) {
  const float w = rweight ? rweight[r] : 1.0f;
  return w * ((std::floor(gate_times[r]) == (double)t) ? 1.0f : 0.0f);
}

}  // namespace

extern "C" {

mrg_status mrg_gate_weights(const double *gate_times, const float *rweight, int64_t nreadouts, int nread, int frame,
                            const float *kw, float *kw_out) {
  if (!gate_args_ok(gate_times, nreadouts, nread) || !kw || !kw_out) {
    if (!kw || !kw_out) set_error("null argument");
    return MRG_ERR_INVALID;
  }
  const int64_t M = nreadouts * nread;
  for (int64_t s = 0; s < M; s++) kw_out[s] = kw[s] * frame_weight(gate_times, rweight, s / nread, frame);
  return MRG_OK;
}

mrg_status mrg_pregate(const double *gate_times, const float *rweight, int64_t nreadouts, int nread, int frame,
                       int reset_dens, const float *kx, const float *ky, const float *kz, const float *kw,
                       const void *data, int ncoil, int64_t coil_stride, float *kx_out, float *ky_out, float *kz_out,
                       float *kw_out, void *data_out, int64_t out_stride, int64_t *count) {
  if (!gate_args_ok(gate_times, nreadouts, nread)) return MRG_ERR_INVALID;
  if (!count) {
    set_error("count is NULL");
    return MRG_ERR_INVALID;
  }
  const int64_t M = nreadouts * nread;
  // number_of_points: the samples of this frame (weight > 0)
  int64_t n = 0;
  for (int64_t r = 0; r < nreadouts; r++)
    if (frame_weight(gate_times, rweight, r, frame) > 0.0f) n += nread;
  *count = n;
  const bool want = kx_out || ky_out || kz_out || kw_out || data_out;
  if (!want) return MRG_OK;
  if (!kx || !ky || !kz || !kw || !kx_out || !ky_out || !kz_out || !kw_out || (data_out && !data) ||
      (data && data_out && ncoil < 1) || (data_out && ncoil > 1 && (coil_stride < M || out_stride < n))) {
    set_error("bad pregate output arguments");
    return MRG_ERR_INVALID;
  }
  // Kw_Scale = 1e6 / (float)number_of_points, a double quotient kept in float (src/recon_lib.cpp:710)
  const float kw_scale = (float)(1e6 / (double)(float)n);
  const float2 *d = static_cast<const float2 *>(data);
  float2 *o = static_cast<float2 *>(data_out);
  int64_t p = 0;
  for (int64_t s = 0; s < M; s++) {
    if (!(frame_weight(gate_times, rweight, s / nread, frame) > 0.0f)) continue;
    kx_out[p] = kx[s];
    ky_out[p] = ky[s];
    kz_out[p] = kz[s];
    kw_out[p] = reset_dens ? 1.0f : kw_scale * kw[s];
    if (o)
      for (int c = 0; c < ncoil; c++) o[(int64_t)c * out_stride + p] = d[(int64_t)c * coil_stride + s];
    p++;
  }
  return MRG_OK;
}

}  // extern "C"
