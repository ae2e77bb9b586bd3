// Uses the C++ drop-in classes exactly as recon_lib's CG loop uses gridFFT
// (src/recon_lib.cpp:1614-1622): per coil, backward (E) then forward (E^H) into
// LHS; and the coil-batched class on the same inputs.  Reads a case written by
// the test (raw little-endian arrays), writes the outputs next to it.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "gridfft_gb300.hpp"

using mrg_cxx::cf;

template <typename T>
static std::vector<T> load(const std::string &path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f.read(reinterpret_cast<char *>(v.data()), sizeof(T) * n)) {
    fprintf(stderr, "cannot read %s\n", path.c_str());
    exit(2);
  }
  return v;
}

template <typename T>
static void save(const std::string &path, const std::vector<T> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), sizeof(T) * v.size());
}

int main(int argc, char **argv) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s dir N C M\n", argv[0]);
    return 2;
  }
  const std::string d = argv[1];
  const int N = atoi(argv[2]), C = atoi(argv[3]);
  const int64_t M = atoll(argv[4]);
  const size_t n3 = (size_t)N * N * N;
  auto kx = load<float>(d + "/kx.bin", M), ky = load<float>(d + "/ky.bin", M);
  auto kz = load<float>(d + "/kz.bin", M), kw = load<float>(d + "/kw.bin", M);
  auto X = load<cf>(d + "/X.bin", n3);
  auto smaps = load<cf>(d + "/smaps.bin", n3 * C);
  try {
    // per-coil operator, the reference's call pattern
    mrg_cxx::gridFFT g;
    g.overgrid = 1.5f;
    g.kernel_type = mrg_cxx::KAISER_KERNEL;
    g.precalc_gridding(N, N, N);
    printf("S=%d og=[%d,%d) grid_x=%.4f beta=%.4f\n", g.Sx, g.og_sx, g.og_ex, g.grid_x, g.betaX);
    std::vector<cf> lhs(n3, cf(0, 0)), tmp(M);
    for (int c = 0; c < C; c++) {
      g.backward(X.data(), smaps.data() + c * n3, tmp.data(), kx.data(), ky.data(), kz.data(), kw.data(), M);
      g.forward(lhs.data(), smaps.data() + c * n3, tmp.data(), kx.data(), ky.data(), kz.data(), kw.data(), M);
    }
    save(d + "/lhs_percoil.bin", lhs);
    // coil-batched operator with the reference class's defaults (overgrid 1.375,
    // unnormalised FFTs: E and E^H sqrt(Sx Sy Sz) times gridFFT's)
    mrg_cxx::gridFFT_CoilThreaded gb;
    gb.precalc_gridding(N, N, N, C);
    printf("coil-threaded: overgrid=%.3f S=%d %d %d\n", gb.overgrid, gb.Sx, gb.Sy, gb.Sz);
    std::vector<cf> y((size_t)C * M), lhs2(n3, cf(0, 0));
    gb.backward(X.data(), smaps.data(), y.data(), kx.data(), ky.data(), kz.data(), kw.data(), M);
    gb.forward(lhs2.data(), smaps.data(), y.data(), kx.data(), ky.data(), kz.data(), kw.data(), M);
    save(d + "/y_batched.bin", y);
    save(d + "/lhs_batched.bin", lhs2);
    // errors surface as exceptions, not exit()
    try {
      mrg_cxx::gridFFT bad;
      bad.precalc_gridding(0, N, N);
      printf("no exception\n");
      return 1;
    } catch (const std::runtime_error &e) {
      printf("caught: %s\n", e.what());
    }
  } catch (const std::exception &e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  printf("ok\n");
  return 0;
}
