// Host-side plan geometry: grid size, crop, Kaiser-Bessel (or triangle / sinc /
// polynomial) lookup table and deapodisation windows.  These are set-up tables
// computed once per plan with the formulas and float/double promotions of
// gridFFT::precalc_kernel and gridFFT::precalc_gridding
// (src/gridFFT.cpp:276-643), so the tables match the reference's bit for bit
// when compiled without floating-point contraction.
#include <algorithm>
#include <cmath>

#include "mrg_internal.h"

namespace mrg {

static const double kRefPI = 3.14159265359;  // src/gridFFT.h:24

// I0 by the Abramowitz & Stegun 9.8.1/9.8.2 polynomials, in the reference's
// float/double mix (src/gridFFT.cpp:1325-1352).
static float bessel_i0(float x) {
  float ax, ans;
  double y;
  if ((ax = std::fabs(x)) < 3.75f) {
    y = x / 3.75;
    y *= y;
    ans = (float)(1.0 + y * (3.5156229 + y * (3.0899424 + y * (1.2067492 + y * (0.2659732 + y * (0.360768e-1 + y * 0.45813e-2))))));
  } else {
    y = 3.75 / ax;
    ans = (float)((std::exp((double)ax) / std::sqrt((double)ax)) *
                  (0.39894228 + y * (0.1328592e-1 + y * (0.225319e-2 + y * (-0.157565e-2 + y * (0.916281e-2 + y * (-0.2057706e-1 + y * (0.2635537e-1 + y * (-0.1647633e-1 + y * 0.392377e-2)))))))));
  }
  return ans;
}

void build_geometry(Geometry &g, const mrg_config &cfg, int Nx, int Ny, int Nz) {
  g.N[0] = Nx;
  g.N[1] = Ny;
  g.N[2] = Nz;
  g.k_rad = cfg.k_rad;
  g.kernel_type = cfg.kernel_type;
  for (int d = 0; d < 3; d++) {
    // rounded gridding ratio: S is a multiple of 16 (src/gridFFT.cpp:500-527)
    g.grid[d] = (float)(16.0 * std::ceil((cfg.overgrid * (float)g.N[d]) / 16.0) / (float)g.N[d]);
    g.S[d] = (int)(g.grid[d] * g.N[d]);
    g.og[d] = (int)((float)g.N[d] * (g.grid[d] - 1) / 2.0);  // src/gridFFT.cpp:536-541
  }
  for (int d = 0; d < 3; d++) {
    g.grid_mod[d] = 600;  // table points per grid unit (src/gridFFT.cpp:278-280)
    float dw = cfg.dwin;
    if (dw == -1) dw = (cfg.kernel_type == MRG_KERNEL_TRIANGLE) ? 1.0f : (cfg.kernel_type == MRG_KERNEL_POLY ? 2.0f : 2.5f);
    g.dwin[d] = dw;
    const int glen = (int)((float)dw * (float)g.grid_mod[d]);
    g.lut_len = glen + 10;
    std::vector<float> &f = g.lut[d];
    f.assign(glen + 10, 0.0f);
    g.beta[d] = 12.0f;  // gridFFT's betaX/Y/Z default, kept by the kernels other than Kaiser-Bessel
    switch (cfg.kernel_type) {
      case MRG_KERNEL_TRIANGLE:
        for (int i = 0; i < glen + 1; i++) f[i] = 1.0f - (float)i / (float)glen;
        break;
      case MRG_KERNEL_SINC:
        for (int i = 0; i < glen + 1; i++) {
          const float pos = ((float)i * (float)dw) / ((float)glen);
          // the cut-off compares the float position with the double 0.01, and the Hamming
          // factor multiplies in double (src/gridFFT.cpp:409-417)
          f[i] = (pos < 0.01) ? 1.0f : (float)(std::sin(pos * kRefPI) / (pos * kRefPI));
          f[i] = (float)(f[i] * (0.54 + 0.46 * std::cos(kRefPI * (float)i / ((float)glen))));
        }
        break;
      case MRG_KERNEL_POLY: {
        const int len = glen + 10;
        for (int i = 0; i < len; i++) {
          const double x = double(i) / double(len), x2 = x * x, x3 = x * x2, x4 = x2 * x2, x5 = x * x4;
          f[i] = (float)(1. + 0.04522831 * x - 3.36020304 * x2 + 1.12417012 * x3 + 2.82448025 * x4 - 1.63447764 * x5);
        }
      } break;
      default: {  // Kaiser-Bessel, beta after Beatty et al. (src/gridFFT.cpp:342-381)
        const float a = g.grid[d];
        float beta = (float)(kRefPI * sqrtf((float)((dw * dw) / (a * a) * (a - 0.5) * (a - 0.5) - 0.8)));
        const float bmin = (float)std::sqrt(std::pow(kRefPI * 2 * dw / a, 2.0) - 9.6752);
        beta = (bmin > beta) ? bmin : beta;
        g.beta[d] = beta;
        for (int i = 0; i < glen + 1; i++) {
          const float pos = ((float)i) / ((float)glen);
          const float arg = sqrtf((float)(1.0 - pos * pos));
          f[i] = bessel_i0(beta * arg) / bessel_i0(beta);
        }
      } break;
    }
    // normalise to sum 0.5*grid_mod (src/gridFFT.cpp:470-472); summed in double
    double s = 0.0;
    for (float v : f) s += v;
    const double scale = 0.5 * g.grid_mod[d] / s;
    g.kb_norm[d] = scale;
    for (float &v : f) v = (float)(v * scale);
  }
  // deapodisation windows with the chop sign, 1/S and the crop folded in,
  // normalised by the (signed) maximum (src/gridFFT.cpp:550-631)
  for (int d = 0; d < 3; d++) {
    const int S = g.S[d];
    std::vector<float> &w = g.win[d];
    w.assign(S, 0.0f);
    const int og_e = g.og[d] + g.N[d];
    for (int i = 0; i < S; i++) {
      const float ipos = i - (float)S / 2.0f;
      for (int gp = 0; gp < g.dwin[d] * g.grid_mod[d]; gp++)
        w[i] = (float)(w[i] + 2 * std::cos(2 * kRefPI * ipos * gp / (float)g.grid_mod[d] / (float)S) * g.lut[d][gp]);
      w[i] = (float)g.grid_mod[d] / w[i];
      const float fact = (float)(2 * (i % 2) - 1);
      w[i] *= fact / S;
      w[i] = (float)(w[i] * ((i < g.og[d]) ? 0.0 : 1.0));
      w[i] = (float)(w[i] * ((i > og_e - 1) ? 0.0 : 1.0));
    }
    float mx = w[0];
    for (float v : w) mx = std::max(mx, v);
    for (float &v : w) v /= mx;
  }
}

// glibc random(): r[i] = r[i-3] + r[i-31] (mod 2^32), seeded by the
// Park-Miller LCG from seed 1, first 310 values discarded, output r >> 1.
GlibcRand::GlibcRand() {
  int32_t s[34];
  s[0] = 1;
  for (int i = 1; i < 31; i++) {
    int64_t v = (16807LL * s[i - 1]) % 2147483647LL;
    if (v < 0) v += 2147483647LL;
    s[i] = (int32_t)v;
  }
  for (int i = 31; i < 34; i++) s[i] = s[i - 31];
  for (int i = 0; i < 34; i++) r[i] = (uint32_t)s[i];
  pos = 34;
  skip(310);
}

namespace {

// Polynomials over Z/2^32 modulo x^31 - x^28 - 1, the characteristic polynomial of the
// stream's recurrence s_i = s_{i-31} + s_{i-3}: coefficient k of x^k in c[k].
struct Poly31 {
  uint32_t c[31];
};

Poly31 poly_mulmod(const Poly31 &a, const Poly31 &b) {
  uint32_t t[61] = {0};
  for (int i = 0; i < 31; i++) {
    if (!a.c[i]) continue;
    for (int j = 0; j < 31; j++) t[i + j] += a.c[i] * b.c[j];
  }
  for (int d = 60; d >= 31; d--) {  // x^d = x^(d-31) x^31 = x^(d-3) + x^(d-31)
    t[d - 3] += t[d];
    t[d - 31] += t[d];
  }
  Poly31 out;
  std::copy(t, t + 31, out.c);
  return out;
}

Poly31 poly_times_x(const Poly31 &a) {
  Poly31 out;
  const uint32_t top = a.c[30];
  for (int k = 30; k >= 1; k--) out.c[k] = a.c[k - 1];
  out.c[0] = top;  // x^31 = x^28 + 1
  out.c[28] += top;
  return out;
}

Poly31 poly_xpow(uint64_t e) {
  Poly31 res{}, base{};
  res.c[0] = 1;
  base.c[1] = 1;
  for (; e; e >>= 1) {
    if (e & 1) res = poly_mulmod(res, base);
    base = poly_mulmod(base, base);
  }
  return res;
}

}  // namespace

// Advances the stream by n draws.  Long skips jump: every later value is a fixed linear
// combination of the last 31, s_{j+e} = sum_k c_k s_{j+k} with x^e = sum_k c_k x^k modulo
// the characteristic polynomial, so the new 34-value window costs O(log n) polynomial
// products instead of n steps.
void GlibcRand::skip(int64_t n) {
  if (n <= 0) return;
  if (n < 64) {
    for (int64_t k = 0; k < n; k++) {
      r[pos % 34] = r[(pos - 31) % 34] + r[(pos - 3) % 34];
      pos++;
    }
    pos = 34 + pos % 34;  // only the position modulo 34 matters; keep it far from overflow
    return;
  }
  const int64_t j = pos - 31;  // s_j .. s_{j+30} are the last 31 values
  uint32_t base[31];
  for (int k = 0; k < 31; k++) base[k] = r[(j + k) % 34];
  // the new window is s_{pos+n-34} .. s_{pos+n-1}: x^(n-3) .. x^(n+30) relative to s_j, in
  // ring slots (pos + n + t) mod 34, found without forming pos + n
  const int b = (int)((pos % 34 + n % 34) % 34);
  Poly31 p = poly_xpow((uint64_t)n - 3);
  for (int t = 0; t < 34; t++) {
    uint32_t v = 0;
    for (int k = 0; k < 31; k++) v += p.c[k] * base[k];
    r[(b + t) % 34] = v;
    p = poly_times_x(p);
  }
  pos = 34 + b;
}

int GlibcRand::next() {
  const uint32_t v = r[(pos - 31) % 34] + r[(pos - 3) % 34];
  r[pos % 34] = v;
  pos++;
  return (int)(v >> 1);
}

bool config_ok(const mrg_config &cfg, int Nx, int Ny, int Nz) {
  if (Nx <= 0 || Ny <= 0 || Nz <= 0) {
    set_error("sizes must be positive");
    return false;
  }
  if (Nx > 65536 || Ny > 65536 || Nz > 65536) {
    set_error("sizes above 65536");
    return false;
  }
  if (!(cfg.overgrid >= 1.0f && cfg.overgrid <= 8.0f) || !(cfg.dwin == -1.0f || (cfg.dwin > 0.0f && cfg.dwin <= 16.0f)) ||
      cfg.kernel_type < 0 || cfg.kernel_type > 3 || cfg.kernel_eval < 0 || cfg.kernel_eval > 1 ||
      (cfg.kernel_eval == 1 && cfg.kernel_type != MRG_KERNEL_KAISER) || cfg.grid_mode < 0 || cfg.grid_mode > 3 ||
      cfg.fft_norm < 0 || cfg.fft_norm > 1) {
    set_error("bad config");
    return false;
  }
  return true;
}

}  // namespace mrg

extern "C" {

mrg_status mrg_plan_geometry(const mrg_config *cfg_in, int Nx, int Ny, int Nz, int S[3], int og[3], float grid[3],
                             float beta[3], int *lut_len, float *lut, float *win) {
  mrg_config cfg;
  if (cfg_in) cfg = *cfg_in; else mrg_config_default(&cfg);
  if (!mrg::config_ok(cfg, Nx, Ny, Nz)) return MRG_ERR_INVALID;
  mrg::Geometry g;
  mrg::build_geometry(g, cfg, Nx, Ny, Nz);
  size_t o = 0;
  for (int d = 0; d < 3; d++) {
    if (S) S[d] = g.S[d];
    if (og) og[d] = g.og[d];
    if (grid) grid[d] = g.grid[d];
    if (beta) beta[d] = g.beta[d];
    if (lut) std::copy(g.lut[d].begin(), g.lut[d].end(), lut + (size_t)d * g.lut_len);
    if (win) std::copy(g.win[d].begin(), g.win[d].end(), win + o);
    o += g.S[d];
  }
  if (lut_len) *lut_len = g.lut_len;
  return MRG_OK;
}

mrg_status mrg_rand_stream(int64_t skip, int n, int *out) {
  if (n < 0 || skip < 0 || (n > 0 && !out)) {
    mrg::set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  mrg::GlibcRand r;
  r.skip(skip);
  for (int i = 0; i < n; i++) out[i] = r.next();
  return MRG_OK;
}

}  // extern "C"
