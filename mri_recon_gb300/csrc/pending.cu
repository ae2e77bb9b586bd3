// Entry points whose kernels are not built yet: they fail loudly.
#include "mrg_internal.h"

static mrg_status pending(const char *what) {
  mrg::set_error(std::string(what) + " is not implemented in this build");
  return MRG_ERR_UNSUPPORTED;
}

extern "C" {
mrg_status mrg_fista(mrg_plan *, const mrg_fista_params *, void *, double *, float *, int, void *) { return pending("mrg_fista"); }
mrg_status mrg_wavelet(void *, int, int, int, int, const int *, const int *, int, int, void *) { return pending("mrg_wavelet"); }
mrg_status mrg_fraction_threshold(const void *, int, int64_t, float, float *, void *) { return pending("mrg_fraction_threshold"); }
mrg_status mrg_soft_threshold(void *, int64_t, float, void *) { return pending("mrg_soft_threshold"); }
mrg_status mrg_llr_update_threshold(const void *, int, int, int, int, const int *, float, float, int, float *, void *) { return pending("mrg_llr_update_threshold"); }
mrg_status mrg_llr_thresh(void *, int, int, int, int, const int *, int, float, float, int64_t, void *) { return pending("mrg_llr_thresh"); }
}
