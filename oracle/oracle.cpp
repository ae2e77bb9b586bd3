// ===========================================================================
// ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the uwmri/mri_recon gridFFT / recon_lib hot path, used
// only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
// the checker.  Nothing in the product (mri_recon_gb300/) links or calls it.
//
// Parity unpinned: the reference ships no golden vectors or known-answer tests
// for this path and cannot be built here (it needs Blitz++ 0.10, FFTW 3.3.6-pl2,
// Armadillo 9.800.2 and HDF5, none of which are present).  Sub-pieces are pinned
// against independent implementations instead (numpy.fft for the FFT, the glibc
// rand() stream, the closed-form Daubechies-4 filters, scipy's I0).
//
// Two precisions share one template:
//   R = float  : mirrors the reference's FP32 arithmetic, including its
//                float/double promotions (e.g. `(1.0 - dz)` in the tap weights).
//   R = double : FP64 twin of the same algorithm (same float LUT and windows).
//
// Layouts: images are column-major x-fastest (index x + Nx*(y + Ny*z)), i.e. a
// C-ordered (Nz, Ny, Nx) numpy array.  k-space samples are flat arrays of M.
// ===========================================================================
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

template <typename R>
using cx = std::complex<R>;

static const double kPI = 3.14159265359;  // gridFFT.h:24 (the reference's PI)

enum { K_TRIANGLE = 0, K_KAISER = 1, K_SINC = 2, K_POLY = 3 };  // gridFFT.h:19-22

// ---------------------------------------------------------------------------
// bessi0: polynomial I0 approximation (Abramowitz & Stegun 9.8.1 / 9.8.2), in
// the mixed float/double form of gridFFT.cpp:1325-1352.
// ---------------------------------------------------------------------------
static float orc_bessi0(float x) {
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

// ---------------------------------------------------------------------------
// Geometry, kernel LUT and deapodisation windows
// (gridFFT.cpp:276-473 precalc_kernel, :475-643 precalc_gridding).
// ---------------------------------------------------------------------------
struct Geom {
  int N[3], S[3], og_s[3], og_e[3];
  float grid[3], dwin[3], grid_mod[3], beta[3];
  double kb_norm[3];  // LUT normalisation factor (analytic evaluation)
  int eval;           // 0: LUT as the reference, 1: analytic Kaiser-Bessel
  int grid_in[3], fft_in[3];
  float k_rad;
  int lut_len;
  std::vector<float> lut[3];
  std::vector<float> win[3];
};

// I0 by its power series sum_k ((z/2)^k / k!)^2 (double; z <= 20 here).
static double i0_series(double z) {
  const double q = 0.25 * z * z;
  double t = 1.0, s = 1.0;
  for (int k = 1; k < 200; k++) {
    t *= q / ((double)k * (double)k);
    s += t;
    if (t < 1e-18 * s) break;
  }
  return s;
}

static void build_geom(Geom &g, int Nx, int Ny, int Nz, float overgrid, float dwin_in, int ktype, float k_rad,
                       int eval) {
  g.N[0] = Nx; g.N[1] = Ny; g.N[2] = Nz;
  g.k_rad = k_rad;
  g.eval = eval;
  for (int d = 0; d < 3; d++) {
    g.grid_in[d] = 1;  // 3D non-Cartesian (mri_data.cpp:324-325)
    g.fft_in[d] = 1;
    // gridFFT.cpp:500-527
    g.grid[d] = (float)(16.0 * std::ceil((overgrid * (float)g.N[d]) / 16.0) / (float)g.N[d]);
    g.S[d] = (int)(g.grid[d] * g.N[d]);
  }
  // precalc_kernel (gridFFT.cpp:276-473)
  for (int d = 0; d < 3; d++) {
    g.grid_mod[d] = 600;
    float dw = dwin_in;
    if (dw == -1) dw = (ktype == K_TRIANGLE) ? 1.0f : (ktype == K_POLY ? 2.0f : 2.5f);
    g.dwin[d] = dw;
    int glen = (int)((float)dw * (float)g.grid_mod[d]);
    g.lut_len = glen + 10;
    std::vector<float> &f = g.lut[d];
    f.assign(glen + 10, 0.0f);
    g.beta[d] = 12;  // gridFFT() default (gridFFT.cpp:33-35), kept by non-Kaiser kernels
    if (ktype == K_TRIANGLE) {
      for (int i = 0; i < glen + 1; i++) f[i] = 1.0f - (float)i / (float)glen;
    } else if (ktype == K_KAISER) {
      float a = g.grid[d];  // grid_scale = 1
      float beta = (float)(kPI * sqrtf((float)((dw * dw) / (a * a) * (a - 0.5) * (a - 0.5) - 0.8)));
      float bmin = (float)std::sqrt(std::pow(kPI * 2 * dw / a, 2.0) - 9.6752);
      beta = (bmin > beta) ? bmin : beta;
      g.beta[d] = beta;
      for (int i = 0; i < glen + 1; i++) {
        float pos = ((float)i) / ((float)glen);
        float arg = sqrtf((float)(1.0 - pos * pos));
        f[i] = orc_bessi0(beta * arg) / orc_bessi0(beta);
      }
    } else if (ktype == K_SINC) {
      for (int i = 0; i < glen + 1; i++) {
        float pos = ((float)i * (float)dw) / ((float)glen);
        f[i] = (pos < 0.01) ? 1.0f : (float)(std::sin(pos * kPI) / (pos * kPI));  // double 0.01
        f[i] = (float)(f[i] * (0.54 + 0.46 * std::cos(kPI * (float)i / ((float)glen))));   // gridFFT.cpp:409-417
      }
    } else {  // polynomial table (gridFFT.cpp:248-269), filled over the whole length
      int len = glen + 10;
      for (int i = 0; i < len; i++) {
        double x = double(i) / double(len), x2 = x * x, x3 = x * x2, x4 = x2 * x2, x5 = x * x4;
        f[i] = (float)(1. + 0.04522831 * x - 3.36020304 * x2 + 1.12417012 * x3 + 2.82448025 * x4 - 1.63447764 * x5);
      }
    }
    double s = 0;
    for (float v : f) s += v;
    double scale = 0.5 * g.grid_mod[d] / s;
    g.kb_norm[d] = scale;
    for (float &v : f) v = (float)(v * scale);
  }
  // crop (gridFFT.cpp:536-541)
  for (int d = 0; d < 3; d++) {
    g.og_s[d] = (int)((float)g.N[d] * (g.grid[d] - 1) / 2.0);
    g.og_e[d] = g.og_s[d] + g.N[d];
  }
  // deapodisation windows with chop and crop (gridFFT.cpp:550-631)
  for (int d = 0; d < 3; d++) {
    int S = g.S[d];
    std::vector<float> &w = g.win[d];
    w.assign(S, 0.0f);
    for (int i = 0; i < S; i++) {
      float ipos = i - (float)S / 2.0f;
      for (int gp = 0; gp < g.dwin[d] * g.grid_mod[d]; gp++) {
        w[i] = (float)(w[i] + 2 * std::cos(2 * kPI * ipos * gp / (float)g.grid_mod[d] / (float)S) * g.lut[d][gp]);
      }
      w[i] = (float)g.grid_mod[d] / w[i];
      float fact = (float)(2 * (i % 2) - 1);
      w[i] *= fact / S;
      w[i] = (float)(w[i] * ((i < g.og_s[d]) ? 0.0 : 1.0));
      w[i] = (float)(w[i] * ((i > g.og_e[d] - 1) ? 0.0 : 1.0));
    }
    float mx = w[0];
    for (float v : w) mx = std::max(mx, v);
    for (float &v : w) v /= mx;
  }
}

// ---------------------------------------------------------------------------
// Mixed-radix FFT (recursive decimation in time), any length.  Replaces the
// reference's FFTW 1D plans (ArrayTemplates.cpp:298-309).  sign = -1 is
// FFTW_FORWARD, +1 is FFTW_BACKWARD; unscaled.
// ---------------------------------------------------------------------------
template <typename R>
struct FFT1 {
  int n;
  std::vector<int> fac;
  std::vector<cx<R>> tw;  // exp(sign*2*pi*i*k/n)
  explicit FFT1(int n_, int sign) : n(n_) {
    int m = n;
    for (int p : {4, 2, 3, 5, 7}) while (m % p == 0) { fac.push_back(p); m /= p; }
    for (int p = 11; m > 1; p += 2) while (m % p == 0) { fac.push_back(p); m /= p; }
    tw.resize(n);
    for (int k = 0; k < n; k++) {
      double a = sign * 2.0 * M_PI * (double)k / (double)n;
      tw[k] = cx<R>((R)std::cos(a), (R)std::sin(a));
    }
  }
  // len * ts == n at every level, so the twiddle index r * k * ts stays below n, and the
  // p-point DFT's W_p^(rq) is tw[((r q) mod p) * n / p]; radices 2 and 4 use butterflies.
  void rec(const cx<R> *in, long is, cx<R> *out, int len, int fi, long ts) const {
    if (len == 1) { out[0] = in[0]; return; }
    int p = fac[fi], m = len / p;
    for (int r = 0; r < p; r++) rec(in + r * is, is * p, out + r * m, m, fi + 1, ts * p);
    cx<R> t[64];
    std::vector<cx<R>> tv;
    cx<R> *tp = t;
    if (p > 64) { tv.resize(p); tp = tv.data(); }
    const long np = n / p;
    const R sg = (R)(tw[np].imag() >= 0 ? 1 : -1);  // W_4^1 = sg * i when p == 4
    for (int k = 0; k < m; k++) {
      tp[0] = out[k];
      for (int r = 1; r < p; r++) tp[r] = out[r * m + k] * tw[(long)r * k * ts];
      if (p == 2) {
        out[k] = tp[0] + tp[1];
        out[k + m] = tp[0] - tp[1];
      } else if (p == 4) {
        const cx<R> a = tp[0] + tp[2], b = tp[0] - tp[2], c = tp[1] + tp[3], d0 = tp[1] - tp[3];
        const cx<R> d(-sg * d0.imag(), sg * d0.real());  // (sg i) (t1 - t3)
        out[k] = a + c;
        out[k + m] = b + d;
        out[k + 2 * m] = a - c;
        out[k + 3 * m] = b - d;
      } else {
        for (int q = 0; q < p; q++) {
          cx<R> acc = tp[0];
          for (int r = 1; r < p; r++) acc += tp[r] * tw[((long)r * q % p) * np];
          out[k + m * q] = acc;
        }
      }
    }
  }
  void run(cx<R> *data, cx<R> *work) const {
    std::memcpy(work, data, sizeof(cx<R>) * n);
    rec(work, 1, data, n, 0, 1);
  }
};

// fft3 along one axis of a sub-box of an array with dims (D0,D1,D2), column-major,
// per-axis scale 1/sqrt(N) in float (ArrayTemplates.cpp:276-427, chop = 0).
// The sub-box is [lo0,hi0) x [lo1,hi1) x [lo2,hi2).
template <typename R>
static void fft3_axis(cx<R> *a, const int D[3], int axis, int sign, const int lo[3], const int hi[3]) {
  int N = D[axis];
  FFT1<R> plan(N, sign);
  R scale = (sizeof(R) == 4) ? (R)(1. / std::sqrt((float)N)) : (R)(1.0 / std::sqrt((double)N));
  long st[3] = {1, (long)D[0], (long)D[0] * D[1]};
  int o1 = (axis == 0) ? 1 : 0, o2 = (axis == 2) ? 1 : 2;
  if (axis == 1) { o1 = 0; o2 = 2; }
#pragma omp parallel
  {
    std::vector<cx<R>> buf(N), work(N);
#pragma omp for collapse(2) schedule(static)
    for (int b = lo[o2]; b < hi[o2]; b++) {
      for (int c = lo[o1]; c < hi[o1]; c++) {
        cx<R> *base = a + (long)b * st[o2] + (long)c * st[o1];
        for (int i = 0; i < N; i++) buf[i] = base[(long)i * st[axis]];
        plan.run(buf.data(), work.data());
        for (int i = 0; i < N; i++) base[(long)i * st[axis]] = buf[i] * scale;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Operator (one coil), gridFFT.cpp:645-1322.
// ---------------------------------------------------------------------------
template <typename R>
struct OPlan {
  Geom g;
  std::vector<cx<R>> grid;  // k3d_grid, S0*S1*S2
  long gsize() const { return (long)g.S[0] * g.S[1] * g.S[2]; }
  long isize() const { return (long)g.N[0] * g.N[1] * g.N[2]; }

  // do_fft (gridFFT.cpp:645-671): pruned FFTW_FORWARD, z then y then x.
  void do_fft() {
    int lo[3] = {0, 0, 0}, hi[3] = {g.S[0], g.S[1], g.S[2]};
    int l1[3] = {g.og_s[0], g.og_s[1], 0}, h1[3] = {g.og_e[0] + 1, g.og_e[1] + 1, g.S[2]};
    fft3_axis<R>(grid.data(), g.S, 2, -1, l1, h1);
    int l2[3] = {g.og_s[0], 0, 0}, h2[3] = {g.og_e[0] + 1, g.S[1], g.S[2]};
    fft3_axis<R>(grid.data(), g.S, 1, -1, l2, h2);
    fft3_axis<R>(grid.data(), g.S, 0, -1, lo, hi);
  }
  // do_ifft (gridFFT.cpp:673-711): full FFTW_BACKWARD, x then y then z.
  void do_ifft() {
    int lo[3] = {0, 0, 0}, hi[3] = {g.S[0], g.S[1], g.S[2]};
    fft3_axis<R>(grid.data(), g.S, 0, +1, lo, hi);
    fft3_axis<R>(grid.data(), g.S, 1, +1, lo, hi);
    fft3_axis<R>(grid.data(), g.S, 2, +1, lo, hi);
  }

  // Tap weight along one axis before rounding: LUT linear interpolation in the
  // reference's float/double mix (gridFFT.cpp:1113-1116); the caller applies
  // the running product and the chop sign and rounds once, as the reference.
  inline double tap_raw(int d, R del) const {
    const std::vector<float> &f = g.lut[d];
    if (g.eval == 1) {  // analytic Kaiser-Bessel with the LUT's normalisation
      const double u = (double)del / ((double)g.grid_mod[d] * (double)g.dwin[d]);
      if (u > 1.0) return 0.0;
      const double b = (double)g.beta[d];
      return g.kb_norm[d] * i0_series(b * std::sqrt(1.0 - u * u)) / i0_series(b);
    }
    if (sizeof(R) == 4) {
      float delf = (float)del;
      float dd = delf - (float)((int)delf);
      return f[(int)delf] * (1.0 - dd) + f[(int)delf + 1] * dd;
    } else {
      int i0 = (int)del;
      double dd = (double)del - (double)i0;
      return (double)f[i0] * (1.0 - dd) + (double)f[i0 + 1] * dd;
    }
  }

  // Per-sample tap range along one axis (gridFFT.cpp:1059-1098): returns
  // false when the sample is outside the grid.
  inline bool tap_range(int d, float k, R &dk, int &s, int &e) const {
    float c = (float)(g.S[d] / 2);
    if (sizeof(R) == 4) {
      float dkf = k * g.grid[d] + c;
      dk = dkf;
      s = std::max((int)std::ceil(dkf - g.dwin[d]), 0);
      e = std::min((int)std::floor(dkf + g.dwin[d]), g.S[d] - 1);
    } else {
      dk = (R)k * (R)g.grid[d] + (R)c;
      s = std::max((int)std::ceil(dk - (R)g.dwin[d]), 0);
      e = std::min((int)std::floor(dk + (R)g.dwin[d]), g.S[d] - 1);
    }
    return !(s >= g.S[d] || e < 0);
  }

  // chop_grid_forward (gridFFT.cpp:1009-1164): scatter data*kw*taper.
  void grid_forward(const cx<R> *data, const float *kx, const float *ky, const float *kz, const float *kw, long M) {
    const int Sx = g.S[0], Sy = g.S[1];
    R *gp = reinterpret_cast<R *>(grid.data());
#pragma omp parallel for schedule(dynamic, 4096)
    for (long i = 0; i < M; i++) {
      float kwv = kw[i];
      if (kwv == 0) continue;
      cx<R> temp = data[i];
      temp *= (R)kwv;
      if (temp == cx<R>(0, 0)) continue;
      R dk[3];
      int s[3], e[3];
      float kk[3] = {kx[i], ky[i], kz[i]};
      bool ok = true;
      for (int d = 0; d < 3; d++) ok = ok && tap_range(d, kk[d], dk[d], s[d], e[d]);
      if (!ok) continue;
      if (sizeof(R) == 4) {
        float kr = kk[0] * kk[0] + kk[1] * kk[1] + kk[2] * kk[2];
        temp *= (R)(float)std::exp(-kr / (2.0 * g.k_rad * g.k_rad));
      } else {
        R kr = (R)kk[0] * kk[0] + (R)kk[1] * kk[1] + (R)kk[2] * kk[2];
        temp *= (R)std::exp(-kr / (2.0 * (double)g.k_rad * (double)g.k_rad));
      }
      for (int lz = s[2]; lz <= e[2]; lz++) {
        R wtz = (R)tap_raw(2, std::fabs((R)g.grid_mod[2] * (dk[2] - (R)lz)));
        wtz *= (R)(2 * (lz % 2) - 1);
        for (int ly = s[1]; ly <= e[1]; ly++) {
          R wty = (R)(wtz * tap_raw(1, std::fabs((R)g.grid_mod[1] * (dk[1] - (R)ly))));
          wty *= (R)(2 * (ly % 2) - 1);
          for (int lx = s[0]; lx <= e[0]; lx++) {
            R wtx = (R)(wty * tap_raw(0, std::fabs((R)g.grid_mod[0] * (dk[0] - (R)lx))));
            wtx *= (R)(2 * (lx % 2) - 1);
            cx<R> t2 = wtx * temp;
            long idx = 2 * ((long)lx + (long)Sx * (ly + (long)Sy * lz));
#pragma omp atomic
            gp[idx] += t2.real();
#pragma omp atomic
            gp[idx + 1] += t2.imag();
          }
        }
      }
    }
  }

  // chop_grid_backward (gridFFT.cpp:1166-1322): gather, optional residual.
  void grid_backward(cx<R> *data, const float *kx, const float *ky, const float *kz, const float *kw, long M,
                     const cx<R> *diff) const {
    const int Sx = g.S[0], Sy = g.S[1];
#pragma omp parallel for schedule(dynamic, 4096)
    for (long i = 0; i < M; i++) {
      if (kw[i] == 0) { data[i] = 0; continue; }
      R dk[3];
      int s[3], e[3];
      float kk[3] = {kx[i], ky[i], kz[i]};
      bool ok = true;
      for (int d = 0; d < 3 && ok; d++) ok = tap_range(d, kk[d], dk[d], s[d], e[d]);
      if (!ok) { data[i] = 0; continue; }
      cx<R> temp(0, 0);
      for (int lz = s[2]; lz <= e[2]; lz++) {
        R wtz = (R)tap_raw(2, std::fabs((R)g.grid_mod[2] * (dk[2] - (R)lz)));
        wtz *= (R)(2 * (lz % 2) - 1);
        for (int ly = s[1]; ly <= e[1]; ly++) {
          R wty = (R)(wtz * tap_raw(1, std::fabs((R)g.grid_mod[1] * (dk[1] - (R)ly))));
          wty *= (R)(2 * (ly % 2) - 1);
          for (int lx = s[0]; lx <= e[0]; lx++) {
            R wtx = (R)(wty * tap_raw(0, std::fabs((R)g.grid_mod[0] * (dk[0] - (R)lx))));
            wtx *= (R)(2 * (lx % 2) - 1);
            temp += wtx * grid[(long)lx + (long)Sx * (ly + (long)Sy * lz)];
          }
        }
      }
      data[i] = diff ? temp - diff[i] : temp;
    }
  }

  // set_image (gridFFT.cpp:972-1002) into a zeroed grid.
  void set_image(const cx<R> *X, const cx<R> *smap) {
    std::fill(grid.begin(), grid.end(), cx<R>(0, 0));
    const int Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
#pragma omp parallel for
    for (int k = 0; k < Nz; k++) {
      R wtz = g.win[2][k + g.og_s[2]];
      for (int j = 0; j < Ny; j++) {
        R wty = wtz * (R)g.win[1][j + g.og_s[1]];
        for (int i = 0; i < Nx; i++) {
          R wt = wty * (R)g.win[0][i + g.og_s[0]];
          long ii = i + (long)Nx * (j + (long)Ny * k);
          cx<R> v = wt * X[ii];
          if (smap) v = v * smap[ii];
          grid[(i + g.og_s[0]) + (long)g.S[0] * ((j + g.og_s[1]) + (long)g.S[1] * (k + g.og_s[2]))] = v;
        }
      }
    }
  }

  // accumulate (gridFFT.cpp:926-956): X += win * image * conj(smap).
  void accumulate(cx<R> *X, const cx<R> *smap) const {
    const int Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
#pragma omp parallel for
    for (int k = 0; k < Nz; k++) {
      R wtz = g.win[2][k + g.og_s[2]];
      for (int j = 0; j < Ny; j++) {
        R wty = wtz * (R)g.win[1][j + g.og_s[1]];
        for (int i = 0; i < Nx; i++) {
          R wt = wty * (R)g.win[0][i + g.og_s[0]];
          long ii = i + (long)Nx * (j + (long)Ny * k);
          cx<R> im = grid[(i + g.og_s[0]) + (long)g.S[0] * ((j + g.og_s[1]) + (long)g.S[1] * (k + g.og_s[2]))];
          X[ii] += smap ? wt * im * std::conj(smap[ii]) : wt * im;
        }
      }
    }
  }

  // gridFFT::forward_sos (gridFFT.cpp:722-757): grid, inverse FFT, deapp
  // (:912-924: image *= winz*winy*winx), then X += image * conj(image)
  // (accumulate_sos, :960-970).
  void adjoint_sos(cx<R> *X, const cx<R> *data, const float *kx, const float *ky, const float *kz,
                   const float *kw, long M) {
    std::fill(grid.begin(), grid.end(), cx<R>(0, 0));
    grid_forward(data, kx, ky, kz, kw, M);
    do_ifft();
    const int Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
#pragma omp parallel for
    for (int k = 0; k < Nz; k++) {
      R wtz = g.win[2][k + g.og_s[2]];
      for (int j = 0; j < Ny; j++) {
        R wty = wtz * (R)g.win[1][j + g.og_s[1]];
        for (int i = 0; i < Nx; i++) {
          long ii = i + (long)Nx * (j + (long)Ny * k);
          cx<R> im = grid[(i + g.og_s[0]) + (long)g.S[0] * ((j + g.og_s[1]) + (long)g.S[1] * (k + g.og_s[2]))];
          im *= (R)(wty * (R)g.win[0][i + g.og_s[0]]);
          X[ii] += cx<R>(im.real() * im.real() + im.imag() * im.imag(), (R)0);
        }
      }
    }
  }
  // gridFFT::forward (E^H, gridFFT.cpp:791-812)
  void adjoint(cx<R> *X, const cx<R> *smap, const cx<R> *data, const float *kx, const float *ky, const float *kz,
               const float *kw, long M) {
    std::fill(grid.begin(), grid.end(), cx<R>(0, 0));
    grid_forward(data, kx, ky, kz, kw, M);
    do_ifft();
    accumulate(X, smap);
  }
  // gridFFT::backward / backward_residual (E, gridFFT.cpp:824-876)
  void forward(const cx<R> *X, const cx<R> *smap, cx<R> *data, const float *kx, const float *ky, const float *kz,
               const float *kw, long M, const cx<R> *diff) {
    set_image(X, smap);
    do_fft();
    grid_backward(data, kx, ky, kz, kw, M, diff);
  }
};

// ---------------------------------------------------------------------------
// Coil-map helpers of the low-resolution map estimate (recon_lib.cpp:2694-2950).
// ---------------------------------------------------------------------------
// gaussian_blur_template (ArrayTemplates.cpp:489-601): per axis with sigma > 0,
// kern[t] = exp(-(t - w)^2 / (2 sigma^2)), w = (int)(5 sigma), t = 0..2w,
// normalised to sum 1; output i sums kern[ii - i + w] * in[ii] over
// ii in [max(i - w, 0), min(i + w, n)) -- the upper end is exclusive, so the
// last tap never contributes, as in the reference.
template <typename R>
static void gaussian_blur(cx<R> *X, int Nx, int Ny, int Nz, const float *sig) {
  const int N[3] = {Nx, Ny, Nz};
  const long st[3] = {1, Nx, (long)Nx * Ny};
  for (int d = 0; d < 3; d++) {
    if (!(sig[d] > 0)) continue;
    const int w = (int)(5 * sig[d]);
    std::vector<float> kern(2 * w + 1);
    double tot = 0;
    for (int t = 0; t <= 2 * w; t++) {
      const float a = (float)t - w;
      kern[t] = (float)std::exp(-(a * a) / (2.0 * (double)(sig[d] * sig[d])));
    }
    for (int t = 0; t <= 2 * w; t++) tot += kern[t];
    for (int t = 0; t <= 2 * w; t++) kern[t] = (float)(kern[t] / tot);
    const int n = N[d];
    const int a1 = (d + 1) % 3, a2 = (d + 2) % 3;
    const long nl = (long)N[a1] * N[a2];
#pragma omp parallel for
    for (long l = 0; l < nl; l++) {
      const long b = (l % N[a1]) * st[a1] + (l / N[a1]) * st[a2];
      std::vector<cx<R>> tmp(n);
      for (int i = 0; i < n; i++) tmp[i] = X[b + i * st[d]];
      for (int i = 0; i < n; i++) {
        const int s0 = std::max(i - w, 0), e0 = std::min(i + w, n);
        cx<R> acc(0, 0);
        for (int ii = s0; ii < e0; ii++) acc += (R)kern[ii - (i - w)] * tmp[ii];
        X[b + i * st[d]] = acc;
      }
    }
  }
}

// sos_normalize with smap_thresh == 0 (recon_lib.cpp:3043-3062):
// A_c /= sqrt(sum_c |A_c|^2), the sum taken coil by coil.
template <typename R>
static void sos_normalize(cx<R> **A, int C, long n) {
#pragma omp parallel for
  for (long v = 0; v < n; v++) {
    R sos = 0;
    for (int c = 0; c < C; c++) sos += A[c][v].real() * A[c][v].real() + A[c][v].imag() * A[c][v].imag();
    sos = std::sqrt(sos);
    for (int c = 0; c < C; c++) A[c][v] = cx<R>(A[c][v].real() / sos, A[c][v].imag() / sos);
  }
}

// ---------------------------------------------------------------------------
// Pipe density compensation: RECON::dcf_calc (recon_lib.cpp:854-917) with
// DCFgridFFT (DCFgridFFT.cpp): starting from Kw = 1, `iters` rounds of
//   X = G Kw (real gridding, forward :174-277), Kw2 = G^T X (backward :323-437),
//   Kw = |Kw2| < 1e-3 ? 0 : Kw / Kw2,
// then Kw *= scale^3 (scale_kw :297-321) and Kw = |Kw|.  G uses the polynomial
// kernel table (loadKernelTable :47-66 / loadKernelTable2 :68-84, normalised to
// sum 0.5*600 :150-152) on a real grid of (int)(overgrid*N + 16) points per axis (x's
// extent from Nz and z's from Nx, as recon_lib allocates it),
// without the chop sign, taps ceil(dk - s*dwin) .. floor(dk + s*dwin) clipped,
// s = |k|/128*(acc - 1) + 1.
// ---------------------------------------------------------------------------
struct ODcfParams {
  int iters;
  float dwin, scale, overgrid, acc;
  int kernel;  // 0 POLY_KERNEL, 1 POLY_KERNEL2
};

static void dcf_table(float dwin, int kernel, std::vector<float> &t) {
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

template <typename R>
struct DcfTaps {
  int s[3], e[3];
  float dk[3], sc;
  bool ok;
};

template <typename R>
static DcfTaps<R> dcf_taps(float kx, float ky, float kz, const int *S, float og, float dwin, float acc) {
  DcfTaps<R> t;
  const float kr = std::sqrt(kx * kx + ky * ky + kz * kz);
  t.sc = (float)(kr / 128.0 * (acc - 1) + 1);
  const float k[3] = {kx, ky, kz};
  t.ok = true;
  for (int d = 0; d < 3; d++) {
    const float c = (float)(S[d] / 2);
    t.dk[d] = k[d] * og + c;
    t.s[d] = std::max((int)std::ceil(t.dk[d] - t.sc * dwin), 0);
    t.e[d] = std::min((int)std::floor(t.dk[d] + t.sc * dwin), S[d] - 1);
    if (t.s[d] >= S[d] || t.e[d] < 0) t.ok = false;
  }
  return t;
}

// one axis weight: lut((int)del)*(1 - d) + lut((int)del + 1)*d in double (1.0 is a double)
static inline double dcf_w(const std::vector<float> &lut, float dk, int l, float sc) {
  const float del = std::fabs(600.0f * (dk - (float)l)) / sc;
  const float d = del - (float)((int)del);
  return lut[(int)del] * (1.0 - d) + lut[(int)del + 1] * d;
}

template <typename R>
static void dcf_pipe(const float *kx0, const float *ky0, const float *kz0, long M, const int *N, const ODcfParams &q,
                     float *kw_out) {
  std::vector<float> lut;
  dcf_table(q.dwin, q.kernel, lut);
  // the image of RECON::dcf_calc is (overgrid Nz + 16, overgrid Ny + 16, overgrid Nx + 16)
  // column-major (src/recon_lib.cpp:873-875), read by DCFgridFFT with its first extent as
  // Sx (src/DCFgridFFT.cpp:174-176): the x and z extents are swapped
  int S[3];
  for (int d = 0; d < 3; d++) S[d] = (int)(q.overgrid * N[2 - d] + 16);
  std::vector<float> kx(M), ky(M), kz(M);
  for (long i = 0; i < M; i++) {
    kx[i] = kx0[i] * q.scale;
    ky[i] = ky0[i] * q.scale;
    kz[i] = kz0[i] * q.scale;
  }
  std::vector<R> X((size_t)S[0] * S[1] * S[2]);
  std::vector<R> kw(M, (R)1), kw2(M);
  for (int it = 0; it < q.iters; it++) {
    std::fill(X.begin(), X.end(), (R)0);
    // forward (DCFgridFFT.cpp:174-277): X += w * Kw
    for (long i = 0; i < M; i++) {
      if (kw[i] == (R)0) continue;
      const DcfTaps<R> t = dcf_taps<R>(kx[i], ky[i], kz[i], S, q.overgrid, q.dwin, q.acc);
      if (!t.ok) continue;
      for (int lz = t.s[2]; lz <= t.e[2]; lz++) {
        const R wtz = (R)dcf_w(lut, t.dk[2], lz, t.sc);
        for (int ly = t.s[1]; ly <= t.e[1]; ly++) {
          const R wty = (R)(wtz * dcf_w(lut, t.dk[1], ly, t.sc));
          for (int lx = t.s[0]; lx <= t.e[0]; lx++) {
            const R wtx = (R)(wty * dcf_w(lut, t.dk[0], lx, t.sc));
            X[(size_t)lx + (size_t)S[0] * (ly + (size_t)S[1] * lz)] += wtx * kw[i];
          }
        }
      }
    }
    // backward (DCFgridFFT.cpp:323-437): Kw2 = sum w * X
#pragma omp parallel for
    for (long i = 0; i < M; i++) {
      kw2[i] = 0;
      const DcfTaps<R> t = dcf_taps<R>(kx[i], ky[i], kz[i], S, q.overgrid, q.dwin, q.acc);
      if (!t.ok) continue;
      R acc = 0;
      for (int lz = t.s[2]; lz <= t.e[2]; lz++) {
        const R wtz = (R)dcf_w(lut, t.dk[2], lz, t.sc);
        for (int ly = t.s[1]; ly <= t.e[1]; ly++) {
          const R wty = (R)(wtz * dcf_w(lut, t.dk[1], ly, t.sc));
          for (int lx = t.s[0]; lx <= t.e[0]; lx++) {
            const R wtx = (R)(wty * dcf_w(lut, t.dk[0], lx, t.sc));
            acc += wtx * X[(size_t)lx + (size_t)S[0] * (ly + (size_t)S[1] * lz)];
          }
        }
      }
      kw2[i] = acc;
    }
    // update (recon_lib.cpp:895-905)
    for (long i = 0; i < M; i++) kw[i] = (std::fabs(kw2[i]) < (R)1e-3) ? (R)0 : kw[i] / kw2[i];
  }
  // scale_kw (DCFgridFFT.cpp:297-321) and |Kw|
  for (long i = 0; i < M; i++) {
    const float kr = std::sqrt(kx[i] * kx[i] + ky[i] * ky[i] + kz[i] * kz[i]);
    const float sc = (float)(kr / 128.0 * (q.acc - 1) + 1);
    kw_out[i] = (float)std::fabs((R)(kw[i] * std::pow(sc, 3)));
  }
}

// ---------------------------------------------------------------------------
// glibc random() TYPE_3 stream for the default seed (the additive lagged
// Fibonacci generator r[i] = r[i-3] + r[i-31], output r >> 1, seeded by the
// Park-Miller LCG).  The reference draws its wavelet and block shifts from
// rand() without calling srand (wavelet3D.cpp:443-448, clear.cpp:408-410).
// ---------------------------------------------------------------------------
struct GRand {
  uint32_t r[34];
  int pos;
  explicit GRand(uint32_t seed = 1) {
    int32_t s[34];
    s[0] = (int32_t)seed;
    for (int i = 1; i < 31; i++) {
      int64_t v = (16807LL * s[i - 1]) % 2147483647LL;
      if (v < 0) v += 2147483647LL;
      s[i] = (int32_t)v;
    }
    for (int i = 31; i < 34; i++) s[i] = s[i - 31];
    for (int i = 0; i < 34; i++) r[i] = (uint32_t)s[i];
    pos = 34;
    for (int i = 34; i < 344; i++) step();
  }
  uint32_t step() {
    uint32_t v = r[(pos - 31) % 34] + r[(pos - 3) % 34];
    r[pos % 34] = v;
    pos++;
    if (pos >= 34 * 1000000) pos = 34 + (pos % 34);
    return v;
  }
  int next() { return (int)(step() >> 1); }
};

// ---------------------------------------------------------------------------
// 3D wavelet (wavelet3D.cpp:563-791): separable periodic DWT with shifts.
// ---------------------------------------------------------------------------
struct Wave {
  int N[3], L[3], S[3], max_level, wN;
  float lpf[4], hpf[4], Slpf[4], Shpf[4];
  Wave(int nx, int ny, int nz, const int lev[3], int type) {
    N[0] = nx; N[1] = ny; N[2] = nz;
    for (int d = 0; d < 3; d++) { L[d] = lev[d]; S[d] = 0; }
    if (type == 0) {  // DB2 (Haar), wavelet3D.cpp:122-140
      wN = 2;
      float h = (float)(1.0 / std::sqrt(2.0));
      lpf[0] = h; lpf[1] = h; hpf[0] = -h; hpf[1] = h;
      Slpf[0] = h; Slpf[1] = h; Shpf[0] = h; Shpf[1] = -h;
    } else {  // DB4 closed form; arrangement as wavelet3D.cpp:168-186
      wN = 4;
      double s3 = std::sqrt(3.0), d = 4.0 * std::sqrt(2.0);
      double h0 = (1 + s3) / d, h1 = (3 + s3) / d, h2 = (3 - s3) / d, h3 = (1 - s3) / d;
      lpf[0] = (float)h3; lpf[1] = (float)h2; lpf[2] = (float)h1; lpf[3] = (float)h0;
      hpf[0] = (float)-h0; hpf[1] = (float)h1; hpf[2] = (float)-h2; hpf[3] = (float)h3;
      Slpf[0] = (float)h0; Slpf[1] = (float)h1; Slpf[2] = (float)h2; Slpf[3] = (float)h3;
      Shpf[0] = (float)h3; Shpf[1] = (float)-h2; Shpf[2] = (float)h1; Shpf[3] = (float)-h0;
    }
    // setup_wavelet_directions (wavelet3D.cpp:99-110)
    max_level = 0;
    for (int dd = 0; dd < 3; dd++) {
      while (std::floor(N[dd] / std::pow(2.0, L[dd])) != (N[dd] / std::pow(2.0, L[dd]))) L[dd]--;
      max_level = std::max(max_level, L[dd]);
    }
  }
  template <typename R>
  void w1d(const cx<R> *in, cx<R> *out, int pts, int dir) const {
    for (int p = 0; p < pts / 2; p++) {
      cx<R> a(0, 0), b(0, 0);
      for (int f = 0; f < wN; f++) {
        int c = ((2 * p - f + S[dir]) + pts) % pts;
        a += (R)lpf[f] * in[c];
        b += (R)hpf[f] * in[c];
      }
      out[p] = a;
      out[p + pts / 2] = b;
    }
  }
  template <typename R>
  void iw1d(const cx<R> *in, cx<R> *out, int pts, int dir) const {
    for (int p = 0; p < pts; p++) out[p] = 0;
    for (int p = 0; p < pts / 2; p++)
      for (int f = 0; f < wN; f++) {
        int c = ((2 * p + f - wN + 1 + S[dir]) + pts) % pts;
        out[c] += in[p] * (R)Slpf[f];
        out[c] += in[p + pts / 2] * (R)Shpf[f];
      }
  }
  template <typename R>
  void axis(cx<R> *X, int Lz, int Ly, int Lx, int ax, int inv) const {
    long sx = 1, sy = N[0], sz = (long)N[0] * N[1];
    int Ls[3] = {Lx, Ly, Lz};
    long st[3] = {sx, sy, sz};
    int n = Ls[ax];
    int a1 = (ax == 0) ? 1 : 0, a2 = (ax == 2) ? 1 : 2;
#pragma omp parallel
    {
      std::vector<cx<R>> b1(n), b2(n);
#pragma omp for collapse(2)
      for (int q = 0; q < Ls[a2]; q++)
        for (int p = 0; p < Ls[a1]; p++) {
          cx<R> *base = X + q * st[a2] + p * st[a1];
          for (int i = 0; i < n; i++) b1[i] = base[i * st[ax]];
          if (inv) iw1d(b1.data(), b2.data(), n, ax); else w1d(b1.data(), b2.data(), n, ax);
          for (int i = 0; i < n; i++) base[i * st[ax]] = b2[i];
        }
    }
  }
  template <typename R>
  void forward(cx<R> *X) const {
    int sz = N[2], sy = N[1], sx = N[0];
    for (int l = 0; l < max_level; l++) {
      if (l < L[0]) axis(X, sz, sy, sx, 0, 0);
      if (l < L[1]) axis(X, sz, sy, sx, 1, 0);
      if (l < L[2]) axis(X, sz, sy, sx, 2, 0);
      if (l < L[2]) sz = N[2] / (int)std::pow(2.0, l + 1);
      if (l < L[1]) sy = N[1] / (int)std::pow(2.0, l + 1);
      if (l < L[0]) sx = N[0] / (int)std::pow(2.0, l + 1);
    }
  }
  template <typename R>
  void backward(cx<R> *X) const {
    int sz = N[2] / (int)std::pow(2.0, L[2]), sy = N[1] / (int)std::pow(2.0, L[1]), sx = N[0] / (int)std::pow(2.0, L[0]);
    for (int l = max_level - 1; l >= 0; l--) {
      if (l < L[2]) sz = N[2] / (int)std::pow(2.0, l);
      if (l < L[1]) sy = N[1] / (int)std::pow(2.0, l);
      if (l < L[0]) sx = N[0] / (int)std::pow(2.0, l);
      if (l < L[2]) axis(X, sz, sy, sx, 2, 1);
      if (l < L[1]) axis(X, sz, sy, sx, 1, 1);
      if (l < L[0]) axis(X, sz, sy, sx, 0, 1);
    }
  }
  void random_shift(GRand &rng) {
    for (int d = 0; d < 3; d++) S[d] = rng.next() % wN;
  }
};

// ---------------------------------------------------------------------------
// Fraction threshold (threshold.cpp:251-391, group_complex = true) and soft
// thresholding (threshold.cpp:766-814).
// ---------------------------------------------------------------------------
template <typename R>
static float get_threshold(cx<R> **vols, int nvol, long nvox, float fraction, double thresh_member) {
  float mx = 0, mn = (float)std::abs(vols[0][0]);
  for (int v = 0; v < nvol; v++)
    for (long i = 0; i < nvox; i++) {
      float a = (float)std::abs(vols[v][i]);
      mx = std::max(mx, a);
      mn = std::min(mn, a);
    }
  long total = (long)nvol * nvox;
  long found = total;
  long target = (long)(fraction * (double)total);
  long acc = (long)(0.001 * (double)total);
  if (target < 2) return 0.0f;
  float value = (float)(0.5 * (mx - mn));
  float max_t = (float)(thresh_member * mx);
  float min_t = mn;
  int iter = 0;
  while ((std::labs(found - target) > acc) && (iter < 64)) {
    if (iter > 0) {
      if (found > target) max_t = value; else min_t = value;
      value = (float)(0.5 * (max_t + min_t));
    }
    iter++;
    found = 0;
    for (int v = 0; v < nvol; v++) {
      long c = 0;
#pragma omp parallel for reduction(+ : c)
      for (long i = 0; i < nvox; i++) c += ((float)std::abs(vols[v][i]) < value) ? 1 : 0;
      found += c;
    }
  }
  return value;
}

template <typename R>
static void soft_threshold(cx<R> *X, long n, float value) {
#pragma omp parallel for
  for (long i = 0; i < n; i++) {
    float cc = (float)std::abs(X[i]);
    if (cc <= value) X[i] = 0;
    else X[i] *= (R)(1.0f - value / cc);
  }
}

// ---------------------------------------------------------------------------
// Locally low rank in time (clear.cpp:233-556, dim = 0, Ne = 1).  SVD by
// one-sided Jacobi in double (the reference uses Armadillo's LAPACK SVD in
// complex<double>; singular values and the thresholded reconstruction are
// unique).
// ---------------------------------------------------------------------------
static void jacobi_svd(std::vector<cx<double>> &A, int m, int n, std::vector<double> &s, std::vector<cx<double>> &V) {
  // A is m x n column-major; on exit A = U*diag(s), V is n x n column-major.
  V.assign((size_t)n * n, 0);
  for (int i = 0; i < n; i++) V[i + (size_t)n * i] = 1;
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        double a = 0, b = 0;
        cx<double> c(0, 0);
        for (int i = 0; i < m; i++) {
          cx<double> x = A[i + (size_t)m * p], y = A[i + (size_t)m * q];
          a += std::norm(x);
          b += std::norm(y);
          c += std::conj(x) * y;
        }
        double ac = std::abs(c);
        if (a == 0 || b == 0 || ac == 0) continue;
        double rel = ac / std::sqrt(a * b);
        off = std::max(off, rel);
        if (rel < 1e-14) continue;
        cx<double> ph = c / ac;  // rotate in the complex plane, then a real Jacobi rotation
        double zeta = (b - a) / (2 * ac);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
        double cs = 1 / std::sqrt(1 + t * t), sn = cs * t;
        for (int i = 0; i < m; i++) {
          cx<double> x = A[i + (size_t)m * p], y = A[i + (size_t)m * q] * std::conj(ph);
          A[i + (size_t)m * p] = cs * x - sn * y;
          A[i + (size_t)m * q] = (sn * x + cs * y) * ph;
        }
        for (int i = 0; i < n; i++) {
          cx<double> x = V[i + (size_t)n * p], y = V[i + (size_t)n * q] * std::conj(ph);
          V[i + (size_t)n * p] = cs * x - sn * y;
          V[i + (size_t)n * q] = (sn * x + cs * y) * ph;
        }
      }
    if (off < 1e-14) break;
  }
  s.assign(n, 0);
  for (int j = 0; j < n; j++) {
    double a = 0;
    for (int i = 0; i < m; i++) a += std::norm(A[i + (size_t)m * j]);
    s[j] = std::sqrt(a);
  }
}

struct LLRParams {
  int bs[3];
  int block_iter;
  float alpha;
  float clear_amp, clear_t2;
};

template <typename R>
static float llr_update_threshold(cx<R> **X, int Nt, const int N[3], LLRParams &p, int iter) {
  for (int d = 0; d < 3; d++) p.bs[d] = std::min(p.bs[d], N[d]);
  int B[3] = {N[0] / p.bs[0], N[1] / p.bs[1], N[2] / p.bs[2]};
  int nb = B[0] * B[1] * B[2];
  int Np = p.bs[0] * p.bs[1] * p.bs[2];
  std::vector<double> sb(nb);
#pragma omp parallel for schedule(dynamic)
  for (int b = 0; b < nb; b++) {
    int bi = b / (B[1] * B[2]), bj = (b / B[2]) % B[1], bk = b % B[2];
    int i0 = bi * p.bs[0], j0 = bj * p.bs[1], k0 = bk * p.bs[2];
    std::vector<cx<double>> A((size_t)Np * Nt), V;
    std::vector<double> s;
    for (int t = 0; t < Nt; t++) {
      int c = 0;
      for (int kk = k0; kk < k0 + p.bs[2]; kk++)
        for (int jj = j0; jj < j0 + p.bs[1]; jj++)
          for (int ii = i0; ii < i0 + p.bs[0]; ii++)
            A[c++ + (size_t)Np * t] = cx<double>(X[t][ii + (long)N[0] * (jj + (long)N[1] * kk)]);
    }
    jacobi_svd(A, Np, Nt, s, V);
    sb[b] = *std::max_element(s.begin(), s.end());
  }
  float amp = 1 + p.clear_amp * std::exp(-((float)iter) / p.clear_t2);
  std::vector<double> nz;
  for (double v : sb) if (v != 0) nz.push_back(v);
  std::sort(nz.begin(), nz.end());
  double med = 0;
  if (!nz.empty()) {
    size_t h = nz.size() / 2;
    med = (nz.size() % 2) ? nz[h] : 0.5 * (nz[h - 1] + nz[h]);
  }
  return (float)(med * amp);
}

template <typename R>
static void llr_thresh(cx<R> **X, int Nt, const int N[3], const LLRParams &p, float smax, GRand &rng) {
  int B[3] = {N[0] / p.bs[0], N[1] / p.bs[1], N[2] / p.bs[2]};
  int nb = B[0] * B[1] * B[2];
  int Np = p.bs[0] * p.bs[1] * p.bs[2];
  double clear_alpha = p.alpha;
  if (clear_alpha == 0.0) return;
  clear_alpha *= smax;
  for (int it = 0; it < p.block_iter; it++) {
    int sh[3];
    for (int d = 0; d < 3; d++) sh[d] = rng.next() % p.bs[d] - p.bs[d] / 2;
    if (p.block_iter == 1) sh[0] = sh[1] = sh[2] = 0;
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < nb; b++) {
      int bi = b / (B[1] * B[2]), bj = (b / B[2]) % B[1], bk = b % B[2];
      int i0 = bi * p.bs[0] + sh[0], j0 = bj * p.bs[1] + sh[1], k0 = bk * p.bs[2] + sh[2];
      std::vector<cx<double>> A((size_t)Np * Nt), A0, V;
      std::vector<double> s;
      std::vector<long> idx(Np);
      int c = 0;
      for (int kk = k0; kk < k0 + p.bs[2]; kk++)
        for (int jj = j0; jj < j0 + p.bs[1]; jj++)
          for (int ii = i0; ii < i0 + p.bs[0]; ii++) {
            int px = (ii + N[0]) % N[0], py = (jj + N[1]) % N[1], pz = (kk + N[2]) % N[2];
            idx[c++] = px + (long)N[0] * (py + (long)N[1] * pz);
          }
      for (int t = 0; t < Nt; t++)
        for (int i = 0; i < Np; i++) A[i + (size_t)Np * t] = cx<double>(X[t][idx[i]]);
      jacobi_svd(A, Np, Nt, s, V);
      // X = U diag(s') V^H with U*diag(s) = A (rotated)
      std::vector<double> f(Nt);
      for (int j = 0; j < Nt; j++) {
        double sp = std::max(s[j] - clear_alpha / p.block_iter, 0.0);
        f[j] = (s[j] > 0) ? sp / s[j] : 0.0;
      }
      for (int i = 0; i < Np; i++)
        for (int t = 0; t < Nt; t++) {
          cx<double> acc(0, 0);
          for (int j = 0; j < Nt; j++) acc += A[i + (size_t)Np * j] * f[j] * std::conj(V[t + (size_t)Nt * j]);
          X[t][idx[i]] = cx<R>((R)acc.real(), (R)acc.imag());
        }
    }
  }
}

// ---------------------------------------------------------------------------
// Coil low rank for CLEAR (clear.cpp:99-232, :561-914 with dim = 2, Ne = 1) on
// per-coil images XX[t*C + c].  A block matrix has Nt*Np rows (frame t, voxel v
// of the block, x fastest: the reference's count) and C columns (coils).
// ---------------------------------------------------------------------------
struct CoilBlocks {
  int bs[3], B[3], nb, Np;
};

static CoilBlocks coil_blocks(const int N[3], const int *bs) {
  CoilBlocks cb;
  for (int d = 0; d < 3; d++) {
    cb.bs[d] = std::min(bs[d], N[d]);  // clear.cpp:109-112
    cb.B[d] = N[d] / cb.bs[d];
  }
  cb.nb = cb.B[0] * cb.B[1] * cb.B[2];
  cb.Np = cb.bs[0] * cb.bs[1] * cb.bs[2];
  return cb;
}

// voxel offsets of block b (i = b % Bx, j = (b / Bx) % By, k = b / (Bx By)) shifted by sh,
// wrapped periodically (clear.cpp:629-648)
static void coil_block_idx(const int N[3], const CoilBlocks &cb, int b, const int sh[3], std::vector<long> &idx) {
  int i0 = (b % cb.B[0]) * cb.bs[0] + sh[0];
  int j0 = ((b / cb.B[0]) % cb.B[1]) * cb.bs[1] + sh[1];
  int k0 = (b / (cb.B[0] * cb.B[1])) * cb.bs[2] + sh[2];
  idx.resize(cb.Np);
  int c = 0;
  for (int kk = k0; kk < k0 + cb.bs[2]; kk++)
    for (int jj = j0; jj < j0 + cb.bs[1]; jj++)
      for (int ii = i0; ii < i0 + cb.bs[0]; ii++) {
        int px = (ii + N[0]) % N[0], py = (jj + N[1]) % N[1], pz = (kk + N[2]) % N[2];
        idx[c++] = px + (long)N[0] * (py + (long)N[1] * pz);
      }
}

// update_threshold(image, 2, iter): the gather writes A(count, t) inside the coil loop
// with count restarting per coil (clear.cpp:185-199), so A holds the last coil's block of
// frame t in column t (Nt <= C, or the reference's column index runs out of range);
// sigma_1 of that A per block, median of the non-zero ones times the amplitude schedule.
template <typename R>
static float coil_update_threshold(cx<R> **XX, int Nt, int C, const int N[3], const int *bs, float amp, float t2,
                                   int iter) {
  const CoilBlocks cb = coil_blocks(N, bs);
  const int R_ = Nt * cb.Np, nt = std::min(Nt, C);
  std::vector<double> sb(cb.nb);
  const int zero[3] = {0, 0, 0};
#pragma omp parallel for schedule(dynamic)
  for (int b = 0; b < cb.nb; b++) {
    std::vector<long> idx;
    coil_block_idx(N, cb, b, zero, idx);
    std::vector<cx<double>> A((size_t)R_ * C, cx<double>(0, 0)), V;
    std::vector<double> sv;
    for (int t = 0; t < nt; t++)
      for (int v = 0; v < cb.Np; v++) A[(t * cb.Np + v) + (size_t)R_ * t] = cx<double>(XX[t * C + C - 1][idx[v]]);
    jacobi_svd(A, R_, C, sv, V);
    sb[b] = *std::max_element(sv.begin(), sv.end());
  }
  float ampv = 1 + amp * std::exp(-((float)iter) / t2);
  std::vector<double> nz;
  for (double v : sb) if (v != 0) nz.push_back(v);
  std::sort(nz.begin(), nz.end());
  double med = 0;
  if (!nz.empty()) {
    size_t h = nz.size() / 2;
    med = (nz.size() % 2) ? nz[h] : 0.5 * (nz[h - 1] + nz[h]);
  }
  return (float)(med * ampv);
}

static void coil_gather(cx<double> *A, int R_, const std::vector<long> &idx, int Np, int Nt, int C, void **XXv, int prec) {
  for (int c = 0; c < C; c++)
    for (int t = 0; t < Nt; t++)
      for (int v = 0; v < Np; v++) {
        const long i = idx[v];
        A[(t * Np + v) + (size_t)R_ * c] = prec ? ((cx<double> **)XXv)[t * C + c][i]
                                                : cx<double>(((cx<float> **)XXv)[t * C + c][i]);
      }
}

// thresh(image, 2) (clear.cpp:561-813): per block iteration three rand() shifts (no
// zero-shift rule here), A = U diag(max(s - alpha smax / block_iter, 0)) V^H.
template <typename R>
static void coil_thresh(cx<R> **XX, int Nt, int C, const int N[3], const int *bs, int block_iter, float alpha,
                        float smax, GRand &rng) {
  const CoilBlocks cb = coil_blocks(N, bs);
  const int R_ = Nt * cb.Np;
  double clear_alpha = alpha;
  if (clear_alpha == 0.0) return;
  clear_alpha *= smax;
  const int prec = sizeof(R) == 8;
  for (int it = 0; it < block_iter; it++) {
    int sh[3];
    for (int d = 0; d < 3; d++) sh[d] = rng.next() % cb.bs[d] - cb.bs[d] / 2;
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < cb.nb; b++) {
      std::vector<long> idx;
      coil_block_idx(N, cb, b, sh, idx);
      std::vector<cx<double>> A((size_t)R_ * C), V;
      std::vector<double> sv;
      coil_gather(A.data(), R_, idx, cb.Np, Nt, C, (void **)XX, prec);
      jacobi_svd(A, R_, C, sv, V);
      std::vector<double> f(C);
      for (int j = 0; j < C; j++) {
        double sp = std::max(sv[j] - clear_alpha / block_iter, 0.0);
        f[j] = (sv[j] > 0) ? sp / sv[j] : 0.0;
      }
      for (int r = 0; r < R_; r++) {
        const int t = r / cb.Np, v = r % cb.Np;
        for (int c = 0; c < C; c++) {
          cx<double> acc(0, 0);
          for (int j = 0; j < C; j++) acc += A[r + (size_t)R_ * j] * f[j] * std::conj(V[c + (size_t)C * j]);
          XX[t * C + c][idx[v]] = cx<R>((R)acc.real(), (R)acc.imag());
        }
      }
    }
  }
}

// combine (clear.cpp:815-914): im = A v1, v1 the right singular vector of the largest
// singular value, here scaled so that its largest-magnitude component is real positive.
template <typename R>
static void coil_combine(cx<R> **XX, int Nt, int C, const int N[3], const int *bs, cx<R> **im) {
  const CoilBlocks cb = coil_blocks(N, bs);
  const int R_ = Nt * cb.Np;
  const int prec = sizeof(R) == 8;
  const int zero[3] = {0, 0, 0};
#pragma omp parallel for schedule(dynamic)
  for (int b = 0; b < cb.nb; b++) {
    std::vector<long> idx;
    coil_block_idx(N, cb, b, zero, idx);
    std::vector<cx<double>> A((size_t)R_ * C), V;
    std::vector<double> sv;
    coil_gather(A.data(), R_, idx, cb.Np, Nt, C, (void **)XX, prec);
    jacobi_svd(A, R_, C, sv, V);  // A = U diag(s)
    int j = (int)(std::max_element(sv.begin(), sv.end()) - sv.begin());
    int m = 0;
    for (int c = 1; c < C; c++)
      if (std::norm(V[c + (size_t)C * j]) > std::norm(V[m + (size_t)C * j])) m = c;
    const cx<double> vm = V[m + (size_t)C * j];
    const cx<double> ph = std::abs(vm) > 0 ? std::conj(vm) / std::abs(vm) : cx<double>(1, 0);
    for (int r = 0; r < R_; r++) {
      const cx<double> a = A[r + (size_t)R_ * j] * ph;  // (A v1)_r = (U s)_r1
      im[r / cb.Np][idx[r % cb.Np]] = cx<R>((R)a.real(), (R)a.imag());
    }
  }
}

// ---------------------------------------------------------------------------
// ESPIRiT coil maps (spirit.cpp:9-66 defaults and init, :137-550), in FP64 from
// the float coil images that gridding.forward leaves in the maps
// (recon_lib.cpp:2892-2899).  kr_f / cr / svd_thresh / shape are the -sp_* flags.
// ---------------------------------------------------------------------------
struct OEspirit {
  float kr_f[3];     // kernel radii (krx_f, kry_f, krz_f)
  int cr[3];         // calibration radii (crx, cry, crz)
  float svd_thresh;  // singular values >= s0 * sqrt(svd_thresh) are kept
  int square;        // 1: SP_SQUARE, 0: SP_CIRCLE
};

static inline double chop_sign(long i) { return (double)(2 * (i % 2) - 1); }

// ifft (ArrayTemplates.cpp:35-88): fftshift (x (2((i+j+k)%2)-1)), FFTW_BACKWARD 3D,
// fftshift, x 1/sqrt(Nz*Ny*Nx) (float)
static void centered_ifft3(std::vector<cx<double>> &a, const int N[3]) {
  const long nx = N[0], ny = N[1], nz = N[2];
  for (long k = 0; k < nz; k++)
    for (long j = 0; j < ny; j++)
      for (long i = 0; i < nx; i++) a[i + nx * (j + ny * k)] *= chop_sign(i + j + k);
  const long st[3] = {1, nx, nx * ny};
  for (int ax = 0; ax < 3; ax++) {
    const int n = N[ax];
    FFT1<double> plan(n, +1);
    std::vector<cx<double>> buf(n), work(n);
    const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
    for (long b = 0; b < N[o2]; b++)
      for (long c = 0; c < N[o1]; c++) {
        cx<double> *base = a.data() + b * st[o2] + c * st[o1];
        for (int i = 0; i < n; i++) buf[i] = base[i * st[ax]];
        plan.run(buf.data(), work.data());
        for (int i = 0; i < n; i++) base[i * st[ax]] = buf[i];
      }
  }
  const double scale = (double)(float)(1.0 / std::sqrt((float)nz * (float)ny * (float)nx));
  for (long k = 0; k < nz; k++)
    for (long j = 0; j < ny; j++)
      for (long i = 0; i < nx; i++) a[i + nx * (j + ny * k)] *= chop_sign(i + j + k) * scale;
}

// rad <= 1 tests of calibrate_ellipsoid (spirit.cpp:199-243, :256-301)
static bool in_acs(int ix, int iy, int iz, const int c[3], bool square) {
  if (square) return true;
  float rad;
  if (c[2] == 0) rad = (float)(ix * ix) / (c[0] * c[0]) + (float)(iy * iy) / (c[1] * c[1]);
  else rad = (float)(ix * ix) / (c[0] * c[0]) + (float)(iy * iy) / (c[1] * c[1]) + (float)(iz * iz) / (c[2] * c[2]);
  return !(rad > 1);
}
static bool in_kernel(int jx, int jy, int jz, const float kf[3], bool square) {
  if (square) return true;
  float krad;
  if (kf[2] == 0) krad = (float)(jx * jx) / (kf[0] * kf[0]) + (float)(jy * jy) / (kf[1] * kf[1]);
  else krad = (float)(jx * jx) / (kf[0] * kf[0]) + (float)(jy * jy) / (kf[1] * kf[1]) + (float)(jz * jz) / (kf[2] * kf[2]);
  return krad <= 1;
}

// Returns nV; maps[c] (N^3 each, x fastest) receive the maps, sv (may be NULL) the
// calibration singular values in descending order (min(rows, cols) of them).
static int espirit(const cx<float> *const *img, int C, const int N[3], const OEspirit &q, cx<double> **maps,
                   double *sv, double *ratio) {
  const long nx = N[0], ny = N[1], nz = N[2], n3 = nx * ny * nz;
  // init (spirit.cpp:36-64)
  float kf[3] = {q.kr_f[0], q.kr_f[1], q.kr_f[2]};
  int kr[3], cr[3];
  for (int d = 0; d < 3; d++) {
    kr[d] = (int)std::ceil(kf[d]);
    cr[d] = q.cr[d];
  }
  if (nz == 1) kr[2] = 0, cr[2] = 0;
  // generateEigenCoils: ifft of each coil image back to k-space (spirit.cpp:146-151)
  std::vector<std::vector<cx<double>>> K(C, std::vector<cx<double>>(n3));
  for (int c = 0; c < C; c++) {
    for (long i = 0; i < n3; i++) K[c][i] = cx<double>(img[c][i]);
    centered_ifft3(K[c], N);
  }
  // calibrate_ellipsoid (spirit.cpp:181-400)
  const int ce[3] = {cr[0] - kr[0], cr[1] - kr[1], cr[2] - kr[2]};
  const long cx0 = nx / 2, cy0 = ny / 2, cz0 = nz / 2;
  struct Off { int x, y, z; };
  std::vector<Off> rows, kpts;
  for (int iz = -ce[2]; iz <= ce[2]; iz++)
    for (int iy = -ce[1]; iy <= ce[1]; iy++)
      for (int ix = -ce[0]; ix <= ce[0]; ix++)
        if (in_acs(ix, iy, iz, ce, q.square)) rows.push_back({ix, iy, iz});
  for (int jz = -kr[2]; jz <= kr[2]; jz++)
    for (int jy = -kr[1]; jy <= kr[1]; jy++)
      for (int jx = -kr[0]; jx <= kr[0]; jx++)
        if (in_kernel(jx, jy, jz, kf, q.square)) kpts.push_back({jx, jy, jz});
  const int m = (int)rows.size(), nk = (int)kpts.size(), n = nk * C;
  std::vector<cx<double>> A((size_t)m * n);  // column-major
  for (int r = 0; r < m; r++)
    for (int c = 0; c < C; c++)
      for (int o = 0; o < nk; o++) {
        const long x = kpts[o].x + rows[r].x + cx0, y = kpts[o].y + rows[r].y + cy0, z = kpts[o].z + rows[r].z + cz0;
        A[r + (size_t)m * (c * nk + o)] = K[c][x + nx * (y + ny * z)];
      }
  // svd_econ(U, s, V, A, "r") by one-sided Jacobi on the columns of A (V accumulated) or,
  // when A has more columns than rows, of A^H (its rotated columns are V diag(s))
  std::vector<double> s;
  std::vector<cx<double>> V;
  const int kmin = std::min(m, n);
  if (m < n) {
    std::vector<cx<double>> B((size_t)n * m), W;
    for (int r = 0; r < m; r++)
      for (int c = 0; c < n; c++) B[c + (size_t)n * r] = std::conj(A[r + (size_t)m * c]);
    jacobi_svd(B, n, m, s, W);
    V.assign((size_t)n * m, cx<double>(0, 0));  // n x m: column j = B_j / s_j
    for (int j = 0; j < m; j++)
      if (s[j] > 0)
        for (int c = 0; c < n; c++) V[c + (size_t)n * j] = B[c + (size_t)n * j] / s[j];
  } else {
    jacobi_svd(A, m, n, s, V);
  }
  std::vector<int> ord(s.size());
  for (int j = 0; j < (int)s.size(); j++) ord[j] = j;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return s[a] > s[b]; });
  const float thresh = (float)(s[ord[0]] * std::sqrt(q.svd_thresh));
  int nV = 0;
  for (int j = 0; j < kmin; j++)
    if (s[ord[j]] >= thresh) nV++;
  if (sv)
    for (int j = 0; j < kmin; j++) sv[j] = s[ord[j]];
  // kernel k(jx, jy, jz, coil, v) over the (2kr+1)^3 box (spirit.cpp:356-392)
  const int bx = 2 * kr[0] + 1, by = 2 * kr[1] + 1, bz = 2 * kr[2] + 1, nb = bx * by * bz;
  std::vector<cx<double>> kern((size_t)nb * C * nV, cx<double>(0, 0));  // [v][c][box]
  for (int v = 0; v < nV; v++)
    for (int c = 0; c < C; c++)
      for (int o = 0; o < nk; o++) {
        const int bi = (kpts[o].x + kr[0]) + bx * ((kpts[o].y + kr[1]) + by * (kpts[o].z + kr[2]));
        kern[((size_t)v * C + c) * nb + bi] = V[(size_t)(c * nk + o) + (size_t)n * ord[v]];
      }
  // prep + getcoils (spirit.cpp:402-525): the kernel placed at the centre of each axis and
  // inverse-FFT'd with the chop signs is, per axis, H(x, j) = m(x) m(N/2 + j) e^{2 pi i (N/2+j) x / N} / sqrt(N)
  auto H = [&](int ax, long x, int j) -> cx<double> {
    const long NN = N[ax], nn = NN / 2 + j;
    const double sc = (double)(float)(1. / std::sqrt((float)NN));
    const double a = 2.0 * M_PI * (double)((nn * x) % NN) / (double)NN;
    return cx<double>(std::cos(a), std::sin(a)) * (chop_sign(x) * chop_sign(nn) * sc);
  };
#pragma omp parallel
  {
    std::vector<cx<double>> Ax((size_t)C * nV), Bh((size_t)nV * C), Vb;
    std::vector<double> sb;
#pragma omp for collapse(2) schedule(dynamic)
    for (long z = 0; z < nz; z++)
      for (long y = 0; y < ny; y++)
        for (long x = 0; x < nx; x++) {
          std::fill(Ax.begin(), Ax.end(), cx<double>(0, 0));
          for (int jz = -kr[2]; jz <= kr[2]; jz++) {
            const cx<double> hz = H(2, z, jz);
            for (int jy = -kr[1]; jy <= kr[1]; jy++) {
              const cx<double> hzy = hz * H(1, y, jy);
              for (int jx = -kr[0]; jx <= kr[0]; jx++) {
                const cx<double> h = hzy * H(0, x, jx);
                const int bi = (jx + kr[0]) + bx * ((jy + kr[1]) + by * (jz + kr[2]));
                for (int v = 0; v < nV; v++)
                  for (int c = 0; c < C; c++) Ax[c + (size_t)C * v] += h * kern[((size_t)v * C + c) * nb + bi];
              }
            }
          }
          // svd_econ(U, s, V, A, "left"): U(:, 0) is the right singular vector of A^H
          for (int v = 0; v < nV; v++)
            for (int c = 0; c < C; c++) Bh[v + (size_t)nV * c] = std::conj(Ax[c + (size_t)C * v]);
          jacobi_svd(Bh, nV, C, sb, Vb);
          const int j0 = (int)(std::max_element(sb.begin(), sb.end()) - sb.begin());
          if (ratio) {  // (s_2 / s_1)^2: the eigenvalue ratio that decides how well u is defined
            double s2 = 0;
            for (int j = 0; j < C; j++)
              if (j != j0) s2 = std::max(s2, sb[j]);
            ratio[x + nx * (y + ny * z)] = sb[j0] > 0 ? (s2 / sb[j0]) * (s2 / sb[j0]) : 1.0;
          }
          // LR(c) = conj(U(c, 0)); phase_correct (spirit.cpp:527-550)
          const long vi = x + nx * (y + ny * z);
          double mag = 0;
          for (int c = 0; c < C; c++) mag += std::norm(Vb[c + (size_t)C * j0]);
          const cx<double> m0 = std::conj(Vb[(size_t)C * j0]);
          const cx<double> ci = std::polar(1.0, -std::arg(m0)) / std::sqrt(mag);
          for (int c = 0; c < C; c++) maps[c][vi] = std::conj(Vb[c + (size_t)C * j0]) * ci;
        }
  }
  return nV;
}

// ---------------------------------------------------------------------------
// C ABI for ctypes (tests / bench baseline leg).
// ---------------------------------------------------------------------------
struct OHandle {
  int prec;  // 0 float, 1 double
  OPlan<float> pf;
  OPlan<double> pd;
  Geom &g() { return prec ? pd.g : pf.g; }
};

template <typename R>
static OPlan<R> &P(OHandle *h);
template <>
OPlan<float> &P<float>(OHandle *h) { return h->pf; }
template <>
OPlan<double> &P<double>(OHandle *h) { return h->pd; }

struct OFrames {
  int Nt, C;
  const float **kx, **ky, **kz, **kw;
  const long *M;
  const void **data;   // [t*C + c]
  const void **smaps;  // [c]
};

struct OFistaParams {
  int max_iter;
  int max_eig_iter;
  int cycle_spins;
  int wave_levels[3];
  int wave_type;       // 0 DB2, 1 DB4
  float thresh;        // fraction (-thresh)
  int use_threshold;   // 0 none, 1 fraction, 2 fixed
  int llr_bs[3];
  int llr_block_iter;
  float llr_alpha;     // clear_alpha_time (0 = off)
  float clear_amp, clear_t2;
  long rand_skip;      // rand() draws consumed before the first shift
};

template <typename R>
static void normal_op(OHandle *h, const OFrames &F, int t, const cx<R> *X, cx<R> *out, std::vector<cx<R>> &tmp,
                      bool residual) {
  OPlan<R> &p = P<R>(h);
  long M = F.M[t];
  tmp.resize(M);
  for (int c = 0; c < F.C; c++) {
    const cx<R> *sm = (const cx<R> *)F.smaps[c];
    const cx<R> *d = (const cx<R> *)F.data[t * F.C + c];
    p.forward(X, sm, tmp.data(), F.kx[t], F.ky[t], F.kz[t], F.kw[t], M, residual ? d : nullptr);
    p.adjoint(out, sm, tmp.data(), F.kx[t], F.ky[t], F.kz[t], F.kw[t], M);
  }
}

// The vector part of one CG iteration (recon_lib.cpp:1659-1722) on Nt frames of n voxels
// (Nz planes): alpha = sum|r|^2 / sum p^H L in complex<double> per-z partial sums cast to
// float, X += alpha P, R -= alpha L, beta = sum|r_new|^2 / sum|r|^2, P = R + beta P.
// Returns sum|r_new|^2.
template <typename R>
static double cg_vectors(int Nt, long n, int Nz, cx<R> **X, cx<R> **Rr, cx<R> **Pp, cx<R> *const *L) {
  const long plane = n / Nz;
  std::vector<cx<double>> a_rr(Nz), a_pl(Nz), a_rn(Nz);
  for (int t = 0; t < Nt; t++) {
#pragma omp parallel for
    for (int k = 0; k < Nz; k++)
      for (long q = 0; q < plane; q++) {
        long i = k * plane + q;
        a_rr[k] += (double)(R)std::norm(Rr[t][i]);
        cx<R> pl = std::conj(Pp[t][i]) * L[t][i];
        a_pl[k] += cx<double>(pl.real(), pl.imag());
      }
  }
  cx<double> rr(0, 0), pl(0, 0), rn(0, 0);
  for (int k = 0; k < Nz; k++) { rr += a_rr[k]; pl += a_pl[k]; }
  cx<double> ds = rr / pl;
  cx<R> scale((R)ds.real(), (R)ds.imag());
  for (int t = 0; t < Nt; t++) {
#pragma omp parallel for
    for (int k = 0; k < Nz; k++)
      for (long q = 0; q < plane; q++) {
        long i = k * plane + q;
        X[t][i] += scale * Pp[t][i];
        Rr[t][i] -= scale * L[t][i];
        a_rn[k] += (double)(R)std::norm(Rr[t][i]);
      }
  }
  for (int k = 0; k < Nz; k++) rn += a_rn[k];
  cx<double> d2 = rn / rr;
  cx<R> scale2((R)d2.real(), (R)d2.imag());
  for (int t = 0; t < Nt; t++)
#pragma omp parallel for
    for (long i = 0; i < n; i++) Pp[t][i] = Rr[t][i] + scale2 * Pp[t][i];
  return rn.real();
}

// SENSE-CG (recon_lib.cpp:1523-1759).  X[t] must be zero on entry.
template <typename R>
static void run_cg(OHandle *h, const OFrames &F, int iters, void **Xv, double *resid) {
  OPlan<R> &p = P<R>(h);
  long n = p.isize();
  int Nt = F.Nt, Nz = p.g.N[2];
  long plane = (long)p.g.N[0] * p.g.N[1];
  std::vector<std::vector<cx<R>>> Rr(Nt, std::vector<cx<R>>(n)), Pp(Nt), L(Nt, std::vector<cx<R>>(n));
  std::vector<cx<R>> tmp;
  cx<R> **X = (cx<R> **)Xv;
  for (int t = 0; t < Nt; t++) {
    for (int c = 0; c < F.C; c++)
      p.adjoint(Rr[t].data(), (const cx<R> *)F.smaps[c], (const cx<R> *)F.data[t * F.C + c], F.kx[t], F.ky[t], F.kz[t],
                F.kw[t], F.M[t]);
    Pp[t] = Rr[t];
  }
  std::vector<cx<R> *> xp(Nt), rp(Nt), pp(Nt), lp(Nt);
  for (int t = 0; t < Nt; t++) {
    xp[t] = X[t];
    rp[t] = Rr[t].data();
    pp[t] = Pp[t].data();
    lp[t] = L[t].data();
  }
  (void)plane;
  for (int it = 0; it < iters; it++) {
    for (int t = 0; t < Nt; t++) {
      std::fill(L[t].begin(), L[t].end(), cx<R>(0, 0));
      normal_op<R>(h, F, t, Pp[t].data(), L[t].data(), tmp, false);
    }
    const double rn = cg_vectors<R>(Nt, n, Nz, xp.data(), rp.data(), pp.data(), lp.data());
    if (resid) resid[it] = rn;
  }
}

// FISTA / IST (recon_lib.cpp:1761-2212) with L1 wavelet threshold
// (recon_lib.cpp:2416-2527) and optional LLR in time (recon_lib.cpp:2117-2121).
template <typename R>
static void run_fista(OHandle *h, const OFrames &F, const OFistaParams &q, void **Xv, double *resid, float *step_out,
                      float *thr_out) {
  OPlan<R> &p = P<R>(h);
  long n = p.isize();
  int Nt = F.Nt;
  cx<R> **X = (cx<R> **)Xv;
  std::vector<std::vector<cx<R>>> Rr(Nt, std::vector<cx<R>>(n)), Xo(Nt, std::vector<cx<R>>(n, cx<R>(0, 0)));
  std::vector<cx<R>> tmp;
  GRand rng(1);
  for (long i = 0; i < q.rand_skip; i++) rng.step();
  // Max eigenvalue by power iteration; seed is the constant -0.5-0.5i because
  // std::rand()/RAND_MAX is an integer division (recon_lib.cpp:1809-1811).
  for (int t = 0; t < Nt; t++) std::fill(X[t], X[t] + n, cx<R>((R)-0.5, (R)-0.5));
  cx<R> step(1, 0);
  for (int it = 0; it < q.max_eig_iter; it++) {
    for (int t = 0; t < Nt; t++) {
      std::fill(Rr[t].begin(), Rr[t].end(), cx<R>(0, 0));
      normal_op<R>(h, F, t, X[t], Rr[t].data(), tmp, false);
    }
    double e = 0;
    for (int t = 0; t < Nt; t++) for (long i = 0; i < n; i++) e += (double)(R)std::norm(Rr[t][i]);
    double max_eig = std::sqrt(e);
    cx<R> sc((R)(1. / max_eig), 0);
    for (int t = 0; t < Nt; t++) for (long i = 0; i < n; i++) X[t][i] = sc * Rr[t][i];
    step = cx<R>((R)(1. / max_eig), 0);
  }
  if (step_out) *step_out = (float)step.real();
  for (int t = 0; t < Nt; t++) std::fill(X[t], X[t] + n, cx<R>(0, 0));
  Wave wave(p.g.N[0], p.g.N[1], p.g.N[2], q.wave_levels, q.wave_type);
  LLRParams lp;
  for (int d = 0; d < 3; d++) lp.bs[d] = q.llr_bs[d];
  lp.block_iter = q.llr_block_iter; lp.alpha = q.llr_alpha; lp.clear_amp = q.clear_amp; lp.clear_t2 = q.clear_t2;
  for (int it = 0; it < q.max_iter; it++) {
    // fista_update (recon_lib.cpp:2177-2212)
    R A = (R)(float)(1.0 + (it - 1.0) / (it + 1.0));
    R B = (R)(float)(-(it - 1.0) / (it + 1.0));
    for (int t = 0; t < Nt; t++)
      for (long i = 0; i < n; i++) {
        cx<R> x0 = Xo[t][i], x1 = X[t][i];
        X[t][i] = A * x1 + B * x0;
        Xo[t][i] = x1;
      }
    for (int t = 0; t < Nt; t++) {
      std::fill(Rr[t].begin(), Rr[t].end(), cx<R>(0, 0));
      normal_op<R>(h, F, t, X[t], Rr[t].data(), tmp, true);
    }
    double e = 0;
    for (int t = 0; t < Nt; t++) for (long i = 0; i < n; i++) e += (double)(R)std::norm(Rr[t][i]);
    if (resid) resid[it] = e;
    for (int t = 0; t < Nt; t++)
      for (long i = 0; i < n; i++) X[t][i] -= Rr[t][i] * step;
    if (q.llr_alpha > 0) {
      float smax = llr_update_threshold<R>(X, Nt, p.g.N, lp, it);
      llr_thresh<R>(X, Nt, p.g.N, lp, smax, rng);
    }
    if (q.use_threshold) {
      float thr = 0;
      for (int spin = 0; spin < q.cycle_spins; spin++) {
        wave.random_shift(rng);
        for (int t = 0; t < Nt; t++) wave.forward<R>(X[t]);
        if (spin == 0) {
          const float scale = (float)(1. / (float)q.cycle_spins);
          thr = (q.use_threshold == 2) ? (float)((double)q.thresh * (double)scale)  // TH_FIXED (threshold.cpp:196-198)
                                       : scale * get_threshold<R>(X, Nt, n, q.thresh, q.thresh);
        }
        for (int t = 0; t < Nt; t++) soft_threshold<R>(X[t], n, thr);
        for (int t = 0; t < Nt; t++) wave.backward<R>(X[t]);
      }
      if (thr_out) thr_out[it] = thr;
    }
  }
}

struct OClearParams {
  int max_iter;
  int bs[3];
  int block_iter;
  float alpha_coil;
  float clear_amp, clear_t2;
  float early_stop_thresh;
  int early_stop_range;
  long rand_skip;
  int use_threshold;
  float thresh;
  int cycle_spins;
  int wave_levels[3];
  int wave_type;
};

// CLEAR (recon_lib.cpp:1025-1238): per-coil images XX[t*C + c] from zero; per iteration
//   R_c = E_c^H W (E_c X_c - d_c), P_c = E_c^H W E_c R_c (E_c: gridFFT without maps),
//   scale = sum |R|^2 / sum P conj(R), X_c -= scale R_c, coil low rank;
// then the combine into im[t].  conj_sum (ArrayTemplates.cpp:462-480) sums in complex
// float per z slice; the energy sums float norms in double (ArrayTemplates.hpp:132-150).
template <typename R>
static int run_clear(OHandle *h, const OFrames &F, const OClearParams &q, void **XXv, void **imv, double *resid) {
  OPlan<R> &p = P<R>(h);
  const long n = p.isize();
  const int Nt = F.Nt, C = F.C, Nz = p.g.N[2];
  const long plane = (long)p.g.N[0] * p.g.N[1];
  cx<R> **XX = (cx<R> **)XXv;
  std::vector<std::vector<cx<R>>> RR((size_t)Nt * C, std::vector<cx<R>>(n));
  std::vector<cx<R>> Pm(n), tmp;
  for (int i = 0; i < Nt * C; i++) std::fill(XX[i], XX[i] + n, cx<R>(0, 0));
  GRand rng(1);
  for (long i = 0; i < q.rand_skip; i++) rng.step();
  Wave wave(p.g.N[0], p.g.N[1], p.g.N[2], q.wave_levels, q.wave_type);
  std::vector<float> diffs;
  double error0 = 0.0;
  int done = 0;
  for (int it = 0; it < q.max_iter; it++) {
    cx<double> rhp(0, 0);
    for (int t = 0; t < Nt; t++) {
      const long M = F.M[t];
      tmp.resize(M);
      for (int c = 0; c < C; c++) {
        cx<R> *Rc = RR[(size_t)t * C + c].data();
        p.forward(XX[t * C + c], nullptr, tmp.data(), F.kx[t], F.ky[t], F.kz[t], F.kw[t], M,
                  (const cx<R> *)F.data[t * C + c]);
        std::fill(Rc, Rc + n, cx<R>(0, 0));
        p.adjoint(Rc, nullptr, tmp.data(), F.kx[t], F.ky[t], F.kz[t], F.kw[t], M);
        std::fill(Pm.begin(), Pm.end(), cx<R>(0, 0));
        p.forward(Rc, nullptr, tmp.data(), F.kx[t], F.ky[t], F.kz[t], F.kw[t], M, nullptr);
        p.adjoint(Pm.data(), nullptr, tmp.data(), F.kx[t], F.ky[t], F.kz[t], F.kw[t], M);
        std::vector<cx<R>> st(Nz, cx<R>(0, 0));
#pragma omp parallel for
        for (int k = 0; k < Nz; k++)
          for (long qq = 0; qq < plane; qq++) st[k] += Pm[k * plane + qq] * std::conj(Rc[k * plane + qq]);
        cx<R> sum(0, 0);
        for (int k = 0; k < Nz; k++) sum += st[k];
        rhp += cx<double>(sum.real(), sum.imag());
      }
    }
    double rhr = 0;
    for (auto &v : RR)
      for (long i = 0; i < n; i++) rhr += (double)(R)std::norm(v[i]);
    if (it == 0) error0 = rhr;
    if (resid) resid[it] = rhr;
    const cx<double> sd = cx<double>(rhr, 0) / rhp;
    const cx<R> scale((R)sd.real(), (R)sd.imag());
    for (int i = 0; i < Nt * C; i++)
      for (long j = 0; j < n; j++) {
        RR[i][j] *= scale;
        XX[i][j] -= RR[i][j];
      }
    done = it + 1;
    if (q.use_threshold) {  // L1_threshold(XX(0, all, all)): frame 0's coil images
      float thr = 0;
      for (int spin = 0; spin < q.cycle_spins; spin++) {
        wave.random_shift(rng);
        for (int c = 0; c < C; c++) wave.forward<R>(XX[c]);
        if (spin == 0) thr = (float)(1. / (float)q.cycle_spins) * get_threshold<R>(XX, C, n, q.thresh, q.thresh);
        for (int c = 0; c < C; c++) soft_threshold<R>(XX[c], n, thr);
        for (int c = 0; c < C; c++) wave.backward<R>(XX[c]);
      }
    }
    if (q.alpha_coil != 0.0f) {
      const float smax = coil_update_threshold<R>(XX, Nt, C, p.g.N, q.bs, q.clear_amp, q.clear_t2, it);
      coil_thresh<R>(XX, Nt, C, p.g.N, q.bs, q.block_iter, q.alpha_coil, smax, rng);
    }
    if (q.early_stop_range > 0 && q.early_stop_thresh > 0.0f) {
      diffs.push_back((float)(std::fabs(rhr) / error0));
      if ((int)diffs.size() > q.early_stop_range) diffs.erase(diffs.begin());
      if ((int)diffs.size() == q.early_stop_range) {
        double sm = 0, sq = 0;
        for (float v : diffs) { sm += v; sq += (double)v * v; }
        float mean = (float)(sm / diffs.size());
        float stdev = (float)std::sqrt(sq / diffs.size() - (double)mean * mean);
        if (stdev < q.early_stop_thresh) break;
      }
    }
  }
  cx<R> **im = (cx<R> **)imv;
  for (int t = 0; t < Nt; t++) std::fill(im[t], im[t] + n, cx<R>(0, 0));
  coil_combine<R>(XX, Nt, C, p.g.N, q.bs, im);
  return done;
}

extern "C" {

void *orc_plan_create(int Nx, int Ny, int Nz, float overgrid, float dwin, int ktype, float k_rad, int prec, int eval) {
  OHandle *h = new OHandle();
  h->prec = prec;
  Geom &g = h->g();
  build_geom(g, Nx, Ny, Nz, overgrid, dwin, ktype, k_rad, eval);
  if (prec) h->pd.grid.assign(h->pd.gsize(), 0); else h->pf.grid.assign(h->pf.gsize(), 0);
  return h;
}
void orc_plan_destroy(void *h) { delete (OHandle *)h; }

void orc_plan_info(void *hv, int *S, int *og, float *grid, float *beta, float *dwin, int *lut_len) {
  Geom &g = ((OHandle *)hv)->g();
  for (int d = 0; d < 3; d++) {
    S[d] = g.S[d]; og[d] = g.og_s[d]; grid[d] = g.grid[d]; beta[d] = g.beta[d]; dwin[d] = g.dwin[d];
  }
  *lut_len = g.lut_len;
}
void orc_get_tables(void *hv, float *lut, float *win) {
  Geom &g = ((OHandle *)hv)->g();
  int o = 0;
  for (int d = 0; d < 3; d++) { std::memcpy(lut + (size_t)d * g.lut_len, g.lut[d].data(), 4 * g.lut_len); }
  for (int d = 0; d < 3; d++) { std::memcpy(win + o, g.win[d].data(), 4 * g.S[d]); o += g.S[d]; }
}

void orc_adjoint(void *hv, void *X, const void *smap, const void *data, const float *kx, const float *ky,
                 const float *kz, const float *kw, long M) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) h->pd.adjoint((cx<double> *)X, (const cx<double> *)smap, (const cx<double> *)data, kx, ky, kz, kw, M);
  else h->pf.adjoint((cx<float> *)X, (const cx<float> *)smap, (const cx<float> *)data, kx, ky, kz, kw, M);
}
void orc_adjoint_sos(void *hv, void *X, const void *data, const float *kx, const float *ky, const float *kz,
                     const float *kw, long M) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) h->pd.adjoint_sos((cx<double> *)X, (const cx<double> *)data, kx, ky, kz, kw, M);
  else h->pf.adjoint_sos((cx<float> *)X, (const cx<float> *)data, kx, ky, kz, kw, M);
}
// gridFFT::k_rad is a public field the map estimate changes between calls
// (recon_lib.cpp:2738, :2786).
void orc_set_k_rad(void *hv, float k_rad) { ((OHandle *)hv)->g().k_rad = k_rad; }
void orc_gaussian_blur(void *X, int Nx, int Ny, int Nz, const float *sig, int prec) {
  if (prec) gaussian_blur<double>((cx<double> *)X, Nx, Ny, Nz, sig);
  else gaussian_blur<float>((cx<float> *)X, Nx, Ny, Nz, sig);
}
void orc_sos_normalize(void **A, int C, long n, int prec) {
  if (prec) sos_normalize<double>((cx<double> **)A, C, n);
  else sos_normalize<float>((cx<float> **)A, C, n);
}
void orc_forward(void *hv, const void *X, const void *smap, void *data, const float *kx, const float *ky,
                 const float *kz, const float *kw, long M, const void *diff) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) h->pd.forward((const cx<double> *)X, (const cx<double> *)smap, (cx<double> *)data, kx, ky, kz, kw, M, (const cx<double> *)diff);
  else h->pf.forward((const cx<float> *)X, (const cx<float> *)smap, (cx<float> *)data, kx, ky, kz, kw, M, (const cx<float> *)diff);
}
// Stage access for kernel-level tests: the plan's grid buffer.
void orc_get_grid(void *hv, void *out) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) std::memcpy(out, h->pd.grid.data(), sizeof(cx<double>) * h->pd.gsize());
  else std::memcpy(out, h->pf.grid.data(), sizeof(cx<float>) * h->pf.gsize());
}
void orc_set_grid(void *hv, const void *in) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) std::memcpy(h->pd.grid.data(), in, sizeof(cx<double>) * h->pd.gsize());
  else std::memcpy(h->pf.grid.data(), in, sizeof(cx<float>) * h->pf.gsize());
}
void orc_grid(void *hv, const void *data, const float *kx, const float *ky, const float *kz, const float *kw, long M) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) { std::fill(h->pd.grid.begin(), h->pd.grid.end(), 0); h->pd.grid_forward((const cx<double> *)data, kx, ky, kz, kw, M); }
  else { std::fill(h->pf.grid.begin(), h->pf.grid.end(), 0); h->pf.grid_forward((const cx<float> *)data, kx, ky, kz, kw, M); }
}
void orc_ungrid(void *hv, void *data, const float *kx, const float *ky, const float *kz, const float *kw, long M, const void *diff) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) h->pd.grid_backward((cx<double> *)data, kx, ky, kz, kw, M, (const cx<double> *)diff);
  else h->pf.grid_backward((cx<float> *)data, kx, ky, kz, kw, M, (const cx<float> *)diff);
}
// FP64 sample values at double-precision positions on the plan's current grid
// (after orc_set_image + orc_fft3): the forward of chop_grid_backward without
// the kw test, for finite-difference checks of trajectory gradients.
void orc_values_at(void *hv, const double *kx, const double *ky, const double *kz, long n, void *out) {
  OHandle *h = (OHandle *)hv;
  OPlan<double> &p = h->pd;
  const Geom &g = p.g;
  cx<double> *o = (cx<double> *)out;
#pragma omp parallel for
  for (long i = 0; i < n; i++) {
    const double kk[3] = {kx[i], ky[i], kz[i]};
    double dk[3];
    int s[3], e[3];
    bool ok = true;
    for (int d = 0; d < 3; d++) {
      dk[d] = kk[d] * (double)g.grid[d] + (double)(g.S[d] / 2);
      s[d] = std::max((int)std::ceil(dk[d] - (double)g.dwin[d]), 0);
      e[d] = std::min((int)std::floor(dk[d] + (double)g.dwin[d]), g.S[d] - 1);
      ok = ok && !(s[d] >= g.S[d] || e[d] < 0);
    }
    cx<double> acc(0, 0);
    if (ok)
      for (int lz = s[2]; lz <= e[2]; lz++) {
        double wz = p.tap_raw(2, std::fabs((double)g.grid_mod[2] * (dk[2] - lz))) * (2 * (lz % 2) - 1);
        for (int ly = s[1]; ly <= e[1]; ly++) {
          double wy = wz * p.tap_raw(1, std::fabs((double)g.grid_mod[1] * (dk[1] - ly))) * (2 * (ly % 2) - 1);
          for (int lx = s[0]; lx <= e[0]; lx++) {
            double w = wy * p.tap_raw(0, std::fabs((double)g.grid_mod[0] * (dk[0] - lx))) * (2 * (lx % 2) - 1);
            acc += w * p.grid[(long)lx + (long)g.S[0] * (ly + (long)g.S[1] * lz)];
          }
        }
      }
    o[i] = acc;
  }
}

void orc_set_image(void *hv, const void *X, const void *smap) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) h->pd.set_image((const cx<double> *)X, (const cx<double> *)smap);
  else h->pf.set_image((const cx<float> *)X, (const cx<float> *)smap);
}
void orc_accumulate(void *hv, void *X, const void *smap) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) h->pd.accumulate((cx<double> *)X, (const cx<double> *)smap);
  else h->pf.accumulate((cx<float> *)X, (const cx<float> *)smap);
}
void orc_fft3(void *hv, int dir) {  // dir -1: do_fft, +1: do_ifft
  OHandle *h = (OHandle *)hv;
  if (h->prec) { if (dir < 0) h->pd.do_fft(); else h->pd.do_ifft(); }
  else { if (dir < 0) h->pf.do_fft(); else h->pf.do_ifft(); }
}
void orc_fft1d(int n, void *data, int sign, int prec) {
  if (prec) { FFT1<double> f(n, sign); std::vector<cx<double>> w(n); f.run((cx<double> *)data, w.data()); }
  else { FFT1<float> f(n, sign); std::vector<cx<float>> w(n); f.run((cx<float> *)data, w.data()); }
}

void orc_cg(void *hv, const OFrames *F, int iters, void **X, double *resid) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) run_cg<double>(h, *F, iters, X, resid); else run_cg<float>(h, *F, iters, X, resid);
}
void orc_fista(void *hv, const OFrames *F, const OFistaParams *q, void **X, double *resid, float *step, float *thr) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) run_fista<double>(h, *F, *q, X, resid, step, thr); else run_fista<float>(h, *F, *q, X, resid, step, thr);
}
// E^H W E per frame, summed over coils, accumulated into out.
// GATING::hist_weight (gating.cpp:1130-1139) after the respiratory factor of
// GATING::weight_data (gating.cpp:1080-1094), and RECON::pregate_data (recon_lib.cpp:675-776)
// for one encode and frame: Kweight(i,j,k) = 1 * rweight(j,k) * (floor(gate_times(j,k)) == t),
// the points with Kweight > 0 in (k, j, i) loop order, kw times Kw_Scale = 1e6/(float)count.
// Returns the count; outputs may be NULL (count only).
long orc_pregate(const double *gate_times, const float *rweight, long nreadouts, int nread, int t, int reset_dens,
                 const float *kx, const float *ky, const float *kz, const float *kw, const void *data, int ncoil,
                 long stride, float *kxo, float *kyo, float *kzo, float *kwo, void *datao, long ostride) {
  std::vector<float> Kweight((size_t)nreadouts * nread, 1.0f);
  for (long r = 0; r < nreadouts; r++)
    for (int i = 0; i < nread; i++) {
      float &w = Kweight[(size_t)r * nread + i];
      if (rweight) w *= rweight[r];
      w *= (std::floor(gate_times[r]) == t) ? (1.0) : (0.0);
    }
  int number_of_points = 0;
  for (float w : Kweight)
    if (w > 0) number_of_points++;
  const float Kw_Scale = (1e6 / ((float)number_of_points));
  if (!kxo) return number_of_points;
  const cx<float> *d = (const cx<float> *)data;
  cx<float> *o = (cx<float> *)datao;
  long p = 0;
  for (long s = 0; s < nreadouts * (long)nread; s++) {
    if (!(Kweight[s] > 0)) continue;
    kxo[p] = kx[s];
    kyo[p] = ky[s];
    kzo[p] = kz[s];
    kwo[p] = reset_dens ? 1.0f : Kw_Scale * kw[s];
    for (int c = 0; o && c < ncoil; c++) o[c * ostride + p] = d[c * stride + s];
    p++;
  }
  return number_of_points;
}

// One CG iteration's vector updates on caller images (the CPU baseline's timing of them).
double orc_cg_vectors(int Nt, long n, int Nz, void **X, void **R, void **P, void **L, int prec) {
  if (prec)
    return cg_vectors<double>(Nt, n, Nz, (cx<double> **)X, (cx<double> **)R, (cx<double> **)P, (cx<double> **)L);
  return cg_vectors<float>(Nt, n, Nz, (cx<float> **)X, (cx<float> **)R, (cx<float> **)P, (cx<float> **)L);
}

void orc_normal(void *hv, const OFrames *F, int t, const void *X, void *out) {
  OHandle *h = (OHandle *)hv;
  if (h->prec) { std::vector<cx<double>> tmp; normal_op<double>(h, *F, t, (const cx<double> *)X, (cx<double> *)out, tmp, false); }
  else { std::vector<cx<float>> tmp; normal_op<float>(h, *F, t, (const cx<float> *)X, (cx<float> *)out, tmp, false); }
}

void orc_wavelet(int Nx, int Ny, int Nz, const int *levels, const int *shift, int wtype, void *X, int inverse, int prec) {
  Wave w(Nx, Ny, Nz, levels, wtype);
  for (int d = 0; d < 3; d++) w.S[d] = shift[d];
  if (prec) { if (inverse) w.backward<double>((cx<double> *)X); else w.forward<double>((cx<double> *)X); }
  else { if (inverse) w.backward<float>((cx<float> *)X); else w.forward<float>((cx<float> *)X); }
}
void orc_wavelet_info(int Nx, int Ny, int Nz, const int *levels, int wtype, int *L_out, float *filters) {
  Wave w(Nx, Ny, Nz, levels, wtype);
  for (int d = 0; d < 3; d++) L_out[d] = w.L[d];
  for (int i = 0; i < w.wN; i++) {
    filters[i] = w.lpf[i]; filters[4 + i] = w.hpf[i]; filters[8 + i] = w.Slpf[i]; filters[12 + i] = w.Shpf[i];
  }
}
float orc_fraction_threshold(void **vols, int nvol, long nvox, float fraction, int prec) {
  if (prec) return get_threshold<double>((cx<double> **)vols, nvol, nvox, fraction, fraction);
  return get_threshold<float>((cx<float> **)vols, nvol, nvox, fraction, fraction);
}
void orc_soft_threshold(void *X, long n, float value, int prec) {
  if (prec) soft_threshold<double>((cx<double> *)X, n, value); else soft_threshold<float>((cx<float> *)X, n, value);
}
float orc_llr_update_threshold(void **X, int Nt, const int *N, const int *bs, float amp, float t2, int iter, int prec) {
  LLRParams p;
  for (int d = 0; d < 3; d++) p.bs[d] = bs[d];
  p.block_iter = 1; p.alpha = 0; p.clear_amp = amp; p.clear_t2 = t2;
  if (prec) return llr_update_threshold<double>((cx<double> **)X, Nt, N, p, iter);
  return llr_update_threshold<float>((cx<float> **)X, Nt, N, p, iter);
}
void orc_llr_thresh(void **X, int Nt, const int *N, const int *bs, int block_iter, float alpha, float smax,
                    long rand_skip, int prec) {
  LLRParams p;
  for (int d = 0; d < 3; d++) p.bs[d] = std::min(bs[d], N[d]);
  p.block_iter = block_iter; p.alpha = alpha; p.clear_amp = 0; p.clear_t2 = 1;
  GRand rng(1);
  for (long i = 0; i < rand_skip; i++) rng.step();
  if (prec) llr_thresh<double>((cx<double> **)X, Nt, N, p, smax, rng);
  else llr_thresh<float>((cx<float> **)X, Nt, N, p, smax, rng);
}
void orc_dcf_pipe(const float *kx, const float *ky, const float *kz, long M, int Nx, int Ny, int Nz,
                  const ODcfParams *q, float *kw, int prec) {
  const int N[3] = {Nx, Ny, Nz};
  if (prec) dcf_pipe<double>(kx, ky, kz, M, N, *q, kw);
  else dcf_pipe<float>(kx, ky, kz, M, N, *q, kw);
}
void orc_dcf_table(float dwin, int kernel, float *out, int *len) {
  std::vector<float> t;
  dcf_table(dwin, kernel, t);
  if (out) std::memcpy(out, t.data(), 4 * t.size());
  *len = (int)t.size();
}
void orc_glibc_rand(long skip, int n, int *out) {
  GRand rng(1);
  for (long i = 0; i < skip; i++) rng.step();
  for (int i = 0; i < n; i++) out[i] = rng.next();
}
float orc_clear_update_threshold(void **XX, int Nt, int C, const int *N, const int *bs, float amp, float t2, int iter,
                                 int prec) {
  return prec ? coil_update_threshold<double>((cx<double> **)XX, Nt, C, N, bs, amp, t2, iter)
              : coil_update_threshold<float>((cx<float> **)XX, Nt, C, N, bs, amp, t2, iter);
}
void orc_clear_thresh(void **XX, int Nt, int C, const int *N, const int *bs, int block_iter, float alpha, float smax,
                      long rand_skip, int prec) {
  GRand rng(1);
  for (long i = 0; i < rand_skip; i++) rng.step();
  if (prec) coil_thresh<double>((cx<double> **)XX, Nt, C, N, bs, block_iter, alpha, smax, rng);
  else coil_thresh<float>((cx<float> **)XX, Nt, C, N, bs, block_iter, alpha, smax, rng);
}
void orc_clear_combine(void **XX, int Nt, int C, const int *N, const int *bs, void **im, int prec) {
  if (prec) coil_combine<double>((cx<double> **)XX, Nt, C, N, bs, (cx<double> **)im);
  else coil_combine<float>((cx<float> **)XX, Nt, C, N, bs, (cx<float> **)im);
}
int orc_clear(void *hv, const OFrames *F, const OClearParams *q, void **XX, void **im, double *resid) {
  OHandle *h = (OHandle *)hv;
  return h->prec ? run_clear<double>(h, *F, *q, XX, im, resid) : run_clear<float>(h, *F, *q, XX, im, resid);
}
int orc_espirit(const void **img, int C, const int *N, const float *kr_f, const int *cr, float svd_thresh, int square,
                void **maps, double *sv, double *ratio) {
  OEspirit q;
  for (int d = 0; d < 3; d++) q.kr_f[d] = kr_f[d], q.cr[d] = cr[d];
  q.svd_thresh = svd_thresh;
  q.square = square;
  return espirit((const cx<float> *const *)img, C, N, q, (cx<double> **)maps, sv, ratio);
}
int orc_num_threads(void) { return omp_get_max_threads(); }
}
