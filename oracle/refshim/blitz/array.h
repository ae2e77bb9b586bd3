// Stand-in for the parts of Blitz++ (blitz/array.h) that the reference's gridFFT.cpp,
// gridFFT_CoilThreaded.cpp, ArrayTemplates.cpp, wavelet3D.cpp, threshold.cpp and clear.cpp
// use, so that those files compile unmodified into oracle/_ref (test infrastructure: the
// reference's own code, run as a checker of the oracle restatement; Blitz++ itself is not
// installed here).
//
// Written from Blitz's documented behaviour, not its source:
//   * Array<T,N> is a strided view of a reference-counted block; the copy constructor
//     and reference() share the block, operator= copies elements (shapes must agree);
//   * the default storage is C order (last index fastest); ColumnMajorArray<N> given to
//     setStorage() makes the first index fastest for the next resize();
//   * A(i, j, k) with ints is an element, with Ranges (inclusive bounds, Range::all()) a
//     view; an int among Ranges drops that dimension;
//   * `A op= x` updates each element as `a op= x` in C++ (a float element times a double
//     is computed in double and rounded once), `A = x` fills;
//   * sum() returns double for float and complex<double> for complex<float> arrays (the
//     sum type Blitz's numeric traits give them), max()/min() the element type;
//   * real()/imag()/abs() of an array are arrays (evaluated eagerly here);
//   * the header brings namespace std into the global namespace, as Blitz's own headers
//     do (the reference's files use cout, ofstream, ... unqualified).
// Anything else aborts with a message rather than guessing.
#ifndef ORACLE_REFSHIM_BLITZ_ARRAY_H
#define ORACLE_REFSHIM_BLITZ_ARRAY_H

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <type_traits>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

using namespace std;

namespace blitz {

enum { firstDim = 0, secondDim = 1, thirdDim = 2, fourthDim = 3, fifthDim = 4, sixthDim = 5, seventhDim = 6 };

[[noreturn]] inline void shim_fail(const char *what) {
  std::fprintf(stderr, "blitz stand-in: %s\n", what);
  std::abort();
}

template <int N>
struct ColumnMajorArray {};

class Range {
 public:
  Range() : first_(0), last_(-1), all_(true) {}
  Range(int first, int last) : first_(first), last_(last), all_(false) {}
  static Range all() { return Range(); }
  int first(int extent) const { return all_ ? 0 : (first_ < 0 ? 0 : first_); }
  int last(int extent) const { return all_ ? extent - 1 : last_; }
  int length(int extent) const { return last(extent) - first(extent) + 1; }

 private:
  int first_, last_;
  bool all_;
};

template <typename T, int N>
class TinyVector {
 public:
  TinyVector() {
    for (int i = 0; i < N; i++) v_[i] = T();
  }
  explicit TinyVector(T a) {
    for (int i = 0; i < N; i++) v_[i] = a;
  }
  template <typename... U, typename = typename std::enable_if<sizeof...(U) == N - 1 && (N > 1)>::type>
  TinyVector(T a, U... rest) : v_{a, static_cast<T>(rest)...} {}
  T &operator()(int i) { return v_[i]; }
  const T &operator()(int i) const { return v_[i]; }
  T &operator[](int i) { return v_[i]; }
  const T &operator[](int i) const { return v_[i]; }
  int length() const { return N; }

 private:
  T v_[N];
};

template <typename T, int N>
inline T product(const TinyVector<T, N> &v) {
  T p = 1;
  for (int i = 0; i < N; i++) p *= v(i);
  return p;
}

template <typename T, int N>
inline std::ostream &operator<<(std::ostream &os, const TinyVector<T, N> &v) {
  os << "(";
  for (int i = 0; i < N; i++) os << (i ? "," : "") << v(i);
  return os << ")";
}

template <typename T, int N>
class Array;

template <typename T>
struct is_shim_array : std::false_type {};
template <typename T, int N>
struct is_shim_array<Array<T, N>> : std::true_type {};

template <typename T>
struct SumType {
  typedef T type;
};
template <>
struct SumType<float> {
  typedef double type;
};
template <>
struct SumType<std::complex<float>> {
  typedef std::complex<double> type;
};

template <typename A>
struct is_index_arg : std::integral_constant<bool, std::is_integral<A>::value || std::is_enum<A>::value> {};

template <typename... A>
struct count_ranges;
template <>
struct count_ranges<> {
  static constexpr int value = 0;
};
template <typename H, typename... A>
struct count_ranges<H, A...> {
  static constexpr int value = (std::is_same<typename std::decay<H>::type, Range>::value ? 1 : 0) +
                               count_ranges<A...>::value;
};

template <typename... A>
struct all_index_args;
template <>
struct all_index_args<> : std::true_type {};
template <typename H, typename... A>
struct all_index_args<H, A...>
    : std::integral_constant<bool, is_index_arg<typename std::decay<H>::type>::value && all_index_args<A...>::value> {};

template <typename T, int N>
class Array {
  template <typename U, int M>
  friend class Array;

 public:
  typedef T T_numtype;

  Array() : data_(nullptr), colmajor_(false) {
    for (int d = 0; d < N; d++) {
      ext_[d] = 0;
      str_[d] = 0;
    }
  }
  template <typename... I, typename = typename std::enable_if<sizeof...(I) == N && all_index_args<I...>::value>::type>
  explicit Array(I... n) : Array() {
    int e[N] = {static_cast<int>(n)...};
    alloc(e);
  }
  explicit Array(const TinyVector<int, N> &s) : Array() { resize(s); }
  Array(const TinyVector<int, N> &s, ColumnMajorArray<N>) : Array() {
    colmajor_ = true;
    resize(s);
  }
  // extents followed by the column-major storage order
  template <int M = N, typename = typename std::enable_if<M == 2>::type>
  Array(int n0, int n1, ColumnMajorArray<2>) : Array() {
    colmajor_ = true;
    resize(n0, n1);
  }
  template <int M = N, typename = typename std::enable_if<M == 3>::type>
  Array(int n0, int n1, int n2, ColumnMajorArray<3>) : Array() {
    colmajor_ = true;
    resize(n0, n1, n2);
  }
  // the copy constructor shares the data, as Blitz's does
  Array(const Array &o) = default;

  // element-wise copy into this array's own storage
  Array &operator=(const Array &o) {
    if (this == &o) return *this;
    if (numElements() == 0 && o.numElements() != 0) shim_fail("assignment to an array without storage");
    for (int d = 0; d < N; d++)
      if (ext_[d] != o.ext_[d]) shim_fail("assignment between arrays of different shapes");
    const long n = numElements();
    for (long i = 0; i < n; i++) at_linear(i) = o.at_linear(i);
    return *this;
  }
  template <typename S, typename = typename std::enable_if<!is_shim_array<S>::value>::type>
  Array &operator=(const S &x) {
    const long n = numElements();
    for (long i = 0; i < n; i++) at_linear(i) = x;
    return *this;
  }
#define SHIM_UPDATE(OP)                                                     \
  template <typename S, typename = typename std::enable_if<!is_shim_array<S>::value>::type> \
  Array &operator OP(const S &x) {                                          \
    const long n = numElements();                                           \
    for (long i = 0; i < n; i++) at_linear(i) OP x;                        \
    return *this;                                                           \
  }
  SHIM_UPDATE(*=)
  SHIM_UPDATE(/=)
  SHIM_UPDATE(+=)
  SHIM_UPDATE(-=)
#undef SHIM_UPDATE

  void setStorage(ColumnMajorArray<N>) { colmajor_ = true; }
  void reference(const Array &o) { copy_view(o); }
  void free() { copy_view(Array()); }

  template <typename... I, typename = typename std::enable_if<sizeof...(I) == N && all_index_args<I...>::value>::type>
  void resize(I... n) {
    int e[N] = {static_cast<int>(n)...};
    alloc(e);
  }
  void resize(const TinyVector<int, N> &s) {
    int e[N];
    for (int d = 0; d < N; d++) e[d] = s(d);
    alloc(e);
  }

  // elements
  template <typename... I>
  typename std::enable_if<sizeof...(I) == N && all_index_args<I...>::value, T &>::type operator()(I... i) {
    const long idx[N] = {static_cast<long>(i)...};
    return data_[offset(idx)];
  }
  template <typename... I>
  typename std::enable_if<sizeof...(I) == N && all_index_args<I...>::value, const T &>::type operator()(I... i) const {
    const long idx[N] = {static_cast<long>(i)...};
    return data_[offset(idx)];
  }
  // fewer int indices than the rank: Blitz computes the offset from the indices given, so
  // the others count as 0 (src/clear.cpp:566-568 reads the shape of image(0, 0) of a
  // rank-3 array of images this way)
  template <typename... I>
  typename std::enable_if<(sizeof...(I) >= 2) && (sizeof...(I) < N) && all_index_args<I...>::value, T &>::type
  operator()(I... i) {
    long idx[N] = {static_cast<long>(i)...};
    return data_[offset(idx)];
  }
  T &operator()(const TinyVector<int, N> &i) {
    long idx[N];
    for (int d = 0; d < N; d++) idx[d] = i(d);
    return data_[offset(idx)];
  }
  // views: Ranges keep a dimension, ints drop it
  template <typename... I>
  typename std::enable_if<sizeof...(I) == N && !all_index_args<I...>::value, Array<T, count_ranges<I...>::value>>::type
  operator()(I... args) const {
    constexpr int M = count_ranges<I...>::value;
    Array<T, M> v;
    v.block_ = block_;
    v.colmajor_ = colmajor_;
    T *p = data_;
    int d = 0, m = 0;
    (void)std::initializer_list<int>{(slice_one(args, d, m, p, v), 0)...};
    v.data_ = p;
    return v;
  }

  T *data() { return data_; }
  const T *data() const { return data_; }
  T *dataFirst() { return data_; }
  long numElements() const {
    long n = 1;
    for (int d = 0; d < N; d++) n *= ext_[d];
    return n;
  }
  long size() const { return numElements(); }
  int extent(int d) const { return ext_[d]; }
  int length(int d) const { return ext_[d]; }
  int rows() const { return ext_[0]; }
  int cols() const { return ext_[1]; }
  int depth() const { return ext_[2]; }
  int lbound(int) const { return 0; }
  int ubound(int d) const { return ext_[d] - 1; }
  long stride(int d) const { return str_[d]; }
  static int rank() { return N; }
  TinyVector<int, N> shape() const {
    TinyVector<int, N> s;
    for (int d = 0; d < N; d++) s(d) = ext_[d];
    return s;
  }
  TinyVector<int, N> extent() const { return shape(); }
  bool isStorageContiguous() const {
    int ord[N];
    order(ord);
    long want = 1;
    for (int k = 0; k < N; k++) {
      if (ext_[ord[k]] > 1 && str_[ord[k]] != want) return false;
      want *= ext_[ord[k]];
    }
    return true;
  }

  // iteration in memory order (the fastest-varying dimension first)
  template <typename A, typename R>
  class iter_t {
   public:
    iter_t() : a_(nullptr), i_(0) {}
    iter_t(A *a, long i) : a_(a), i_(i) {}
    R &operator*() const { return a_->at_linear(i_); }
    R *operator->() const { return &a_->at_linear(i_); }
    iter_t &operator++() {
      ++i_;
      return *this;
    }
    iter_t operator++(int) {
      iter_t t = *this;
      ++i_;
      return t;
    }
    bool operator==(const iter_t &o) const { return i_ == o.i_; }
    bool operator!=(const iter_t &o) const { return i_ != o.i_; }

   private:
    A *a_;
    long i_;
  };
  typedef iter_t<Array, T> iterator;
  typedef iter_t<const Array, const T> const_iterator;
  iterator begin() { return iterator(this, 0); }
  iterator end() { return iterator(this, numElements()); }
  const_iterator begin() const { return const_iterator(this, 0); }
  const_iterator end() const { return const_iterator(this, numElements()); }

  // element i of the memory-order walk
  T &at_linear(long i) const {
    int ord[N];
    order(ord);
    long off = 0;
    for (int k = 0; k < N; k++) {
      const int d = ord[k];
      const long q = ext_[d] ? i % ext_[d] : 0;
      i = ext_[d] ? i / ext_[d] : 0;
      off += q * str_[d];
    }
    return data_[off];
  }

 private:
  std::shared_ptr<std::vector<T>> block_;
  T *data_;
  int ext_[N];
  long str_[N];
  bool colmajor_;

  void copy_view(const Array &o) {
    block_ = o.block_;
    data_ = o.data_;
    colmajor_ = o.colmajor_;
    for (int d = 0; d < N; d++) {
      ext_[d] = o.ext_[d];
      str_[d] = o.str_[d];
    }
  }
  void alloc(const int *e) {
    long n = 1;
    for (int d = 0; d < N; d++) {
      if (e[d] < 0) shim_fail("negative extent");
      ext_[d] = e[d];
      n *= e[d];
    }
    block_ = std::make_shared<std::vector<T>>((size_t)n);
    data_ = block_->data();
    long s = 1;
    for (int k = 0; k < N; k++) {
      const int d = colmajor_ ? k : N - 1 - k;
      str_[d] = s;
      s *= ext_[d];
    }
  }
  long offset(const long *idx) const {
    long off = 0;
    for (int d = 0; d < N; d++) {
      if (idx[d] < 0 || idx[d] >= ext_[d]) shim_fail("index out of range");
      off += idx[d] * str_[d];
    }
    return off;
  }
  // dimensions sorted by stride (ties: storage order), fastest first
  void order(int *ord) const {
    for (int d = 0; d < N; d++) ord[d] = colmajor_ ? d : N - 1 - d;
    std::stable_sort(ord, ord + N, [this](int a, int b) { return str_[a] < str_[b]; });
  }
  template <int M>
  void slice_one(const Range &r, int &d, int &m, T *&p, Array<T, M> &v) const {
    const int f = r.first(ext_[d]), l = r.last(ext_[d]);
    if (f < 0 || l >= ext_[d] || l < f - 1) shim_fail("range out of bounds");
    p += (long)f * str_[d];
    v.ext_[m] = l - f + 1;
    v.str_[m] = str_[d];
    ++m;
    ++d;
  }
  template <int M, typename I>
  typename std::enable_if<is_index_arg<I>::value>::type slice_one(I i, int &d, int &m, T *&p, Array<T, M> &) const {
    if ((long)i < 0 || (long)i >= ext_[d]) shim_fail("index out of range in a view");
    p += (long)i * str_[d];
    ++d;
  }
};

template <typename T, int N>
inline std::ostream &operator<<(std::ostream &os, const Array<T, N> &a) {
  os << a.shape() << " [";
  const long n = a.numElements();
  for (long i = 0; i < n && i < 16; i++) os << (i ? " " : "") << a.at_linear(i);
  return os << (n > 16 ? " ...]" : "]");
}

template <typename T, int N>
inline typename SumType<T>::type sum(const Array<T, N> &a) {
  typename SumType<T>::type s = typename SumType<T>::type();
  const long n = a.numElements();
  for (long i = 0; i < n; i++) s += a.at_linear(i);
  return s;
}
template <typename T, int N>
inline T max(const Array<T, N> &a) {
  const long n = a.numElements();
  if (n == 0) shim_fail("max of an empty array");
  T m = a.at_linear(0);
  for (long i = 1; i < n; i++) m = (a.at_linear(i) > m) ? a.at_linear(i) : m;
  return m;
}
template <typename T, int N>
inline T min(const Array<T, N> &a) {
  const long n = a.numElements();
  if (n == 0) shim_fail("min of an empty array");
  T m = a.at_linear(0);
  for (long i = 1; i < n; i++) m = (a.at_linear(i) < m) ? a.at_linear(i) : m;
  return m;
}
template <typename T, int N>
inline typename SumType<T>::type mean(const Array<T, N> &a) {
  return sum(a) / (double)a.numElements();
}

template <typename T, int N, typename F>
inline auto shim_map(const Array<T, N> &a, F f) -> Array<decltype(f(std::declval<T>())), N> {
  Array<decltype(f(std::declval<T>())), N> out(a.shape());
  const long n = a.numElements();
  for (long i = 0; i < n; i++) out.at_linear(i) = f(a.at_linear(i));
  return out;
}
template <typename T, int N>
inline Array<T, N> real(const Array<std::complex<T>, N> &a) {
  return shim_map(a, [](const std::complex<T> &z) { return z.real(); });
}
template <typename T, int N>
inline Array<T, N> imag(const Array<std::complex<T>, N> &a) {
  return shim_map(a, [](const std::complex<T> &z) { return z.imag(); });
}
template <typename T, int N>
inline Array<T, N> abs(const Array<std::complex<T>, N> &a) {
  return shim_map(a, [](const std::complex<T> &z) { return std::abs(z); });
}
template <typename T, int N>
inline Array<std::complex<T>, N> conj(const Array<std::complex<T>, N> &a) {
  return shim_map(a, [](const std::complex<T> &z) { return std::conj(z); });
}

}  // namespace blitz

#endif
