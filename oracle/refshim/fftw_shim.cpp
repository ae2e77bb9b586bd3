// Implementation of the FFTW stand-in (refshim/fftw3.h) for oracle/_ref: complex DFTs of
// any length by recursive mixed-radix decimation in time (smallest prime factor first,
// direct sums for the prime lengths), computed in double precision and rounded to float
// once.  A plan only records sizes, sign and roots of unity, so it can be executed from
// several threads on different arrays (the reference calls fftwf_execute_dft that way).
#include <cmath>
#include <complex>
#include <cstdlib>
#include <vector>

#include "fftw3.h"

typedef std::complex<double> cd;

struct fftwf_plan_s {
  std::vector<int> n;                // dimensions, row-major (the last contiguous)
  int sign;
  std::vector<std::vector<cd>> root;  // per dimension: exp(sign 2 pi i t / n), t < n
  fftwf_complex *in, *out;
};

namespace {

int smallest_factor(int n) {
  for (int p = 2; p * p <= n; p++)
    if (n % p == 0) return p;
  return n;
}

// out[k] = sum_j in[j*stride] w^(j k), n points; w = root table of length N, step N / n.
void dft_rec(const cd *in, long stride, cd *out, int n, const std::vector<cd> &root, int step) {
  const int N = (int)root.size();
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  const int p = smallest_factor(n);
  const int m = n / p;
  if (p == n) {  // prime length: direct sum
    for (int k = 0; k < n; k++) {
      cd s(0.0, 0.0);
      for (int j = 0; j < n; j++) s += in[j * stride] * root[(long)((long)j * k % n) * step % N];
      out[k] = s;
    }
    return;
  }
  // p interleaved sub-sequences of length m, each transformed into out[r*m .. r*m + m)
  std::vector<cd> sub((size_t)n);
  for (int r = 0; r < p; r++) dft_rec(in + r * stride, stride * p, sub.data() + (size_t)r * m, m, root, step * p);
  for (int q = 0; q < p; q++)
    for (int k = 0; k < m; k++) {
      const int kk = k + m * q;
      cd s(0.0, 0.0);
      for (int r = 0; r < p; r++) s += sub[(size_t)r * m + k] * root[(long)((long)r * kk % n) * step % N];
      out[kk] = s;
    }
}

void transform(const fftwf_plan_s *pl, fftwf_complex *in, fftwf_complex *out) {
  long total = 1;
  for (int d : pl->n) total *= d;
  std::vector<cd> a((size_t)total);
  for (long i = 0; i < total; i++) a[i] = cd(in[i][0], in[i][1]);
  long inner = total;
  std::vector<cd> line, res;
  for (size_t ax = 0; ax < pl->n.size(); ax++) {
    const int n = pl->n[ax];
    inner /= n;                       // stride of this axis
    const long outer = total / (inner * n);
    line.resize(n);
    res.resize(n);
    for (long o = 0; o < outer; o++)
      for (long i = 0; i < inner; i++) {
        cd *base = a.data() + o * n * inner + i;
        for (int j = 0; j < n; j++) line[j] = base[(long)j * inner];
        dft_rec(line.data(), 1, res.data(), n, pl->root[ax], 1);
        for (int j = 0; j < n; j++) base[(long)j * inner] = res[j];
      }
  }
  for (long i = 0; i < total; i++) {
    out[i][0] = (float)a[i].real();
    out[i][1] = (float)a[i].imag();
  }
}

fftwf_plan make_plan(int rank, const int *n, fftwf_complex *in, fftwf_complex *out, int sign) {
  fftwf_plan_s *p = new fftwf_plan_s;
  p->n.assign(n, n + rank);
  p->sign = sign;
  p->in = in;
  p->out = out;
  for (int d = 0; d < rank; d++) {
    std::vector<cd> r((size_t)n[d]);
    for (int t = 0; t < n[d]; t++) {
      const double ang = (double)sign * 2.0 * 3.14159265358979323846 * (double)t / (double)n[d];
      r[t] = cd(std::cos(ang), std::sin(ang));
    }
    p->root.push_back(r);
  }
  return p;
}

}  // namespace

extern "C" {

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned) {
  return make_plan(1, &n, in, out, sign);
}
fftwf_plan fftwf_plan_dft_3d(int n0, int n1, int n2, fftwf_complex *in, fftwf_complex *out, int sign, unsigned) {
  const int n[3] = {n0, n1, n2};
  return make_plan(3, n, in, out, sign);
}
fftwf_plan fftwf_plan_dft(int rank, const int *n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned) {
  return make_plan(rank, n, in, out, sign);
}
void fftwf_execute(const fftwf_plan p) { transform(p, p->in, p->out); }
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out) { transform(p, in, out); }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }
void *fftwf_malloc(size_t n) { return std::aligned_alloc(16, (n + 15) / 16 * 16); }
void fftwf_free(void *p) { std::free(p); }
int fftwf_import_wisdom_from_file(FILE *) { return 0; }
void fftwf_export_wisdom_to_file(FILE *) {}
int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int) {}

}  // extern "C"
