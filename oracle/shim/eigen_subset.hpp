// Minimal Eigen-compatible dense matrix, written for this project so that the
// reference optimizer headers (pngf-opt/pngfopt.hpp, pngf-opt/linalg.hpp)
// compile unmodified without Eigen being installed.
//
// Test infrastructure only: this header is used to build the oracle
// (oracle/_ref), never by the product library.
//
// Covers exactly what those headers use:
//   Matrix<T,Rows,Cols> with Dynamic sizes, Vector<T,Dynamic>, column-major
//   storage, data(), resize(), rows()/cols(), (i,j) and linear (i) access,
//   row()/col() proxies with setZero() and +=, setZero() on whole matrices,
//   and matrix*matrix / matrix*vector products.
#pragma once
#include <complex>
#include <cstddef>
#include <vector>

namespace Eigen {

constexpr int Dynamic = -1;

template <typename T, int R, int C> class Matrix;

// Strided view of one row or one column of a column-major matrix.
template <typename T> struct StridedView {
  T *base;
  long n;
  long stride;
  T &operator()(long i) { return base[i * stride]; }
  const T &operator()(long i) const { return base[i * stride]; }
  void setZero() {
    for (long i = 0; i < n; ++i) base[i * stride] = T(0);
  }
  StridedView &operator+=(const StridedView &o) {
    for (long i = 0; i < n; ++i) base[i * stride] += o.base[i * o.stride];
    return *this;
  }
  template <int R2, int C2> StridedView &operator+=(const Matrix<T, R2, C2> &o);
};

template <typename T, int R, int C> class Matrix {
 public:
  Matrix() : nr_(R > 0 ? R : 0), nc_(C > 0 ? C : 0), v_((size_t)nr_ * nc_) {}
  Matrix(long r, long c) : nr_(r), nc_(c), v_((size_t)r * c) {}

  void resize(long r, long c) {
    nr_ = r;
    nc_ = c;
    v_.assign((size_t)r * c, T(0));
  }
  // Vector form: resize(n) keeps the fixed dimension at 1.
  void resize(long n) {
    if (C == 1) resize(n, 1);
    else resize(1, n);
  }
  long rows() const { return nr_; }
  long cols() const { return nc_; }
  long size() const { return nr_ * nc_; }
  T *data() { return v_.data(); }
  const T *data() const { return v_.data(); }

  T &operator()(long i, long j) { return v_[(size_t)i + (size_t)j * nr_]; }
  const T &operator()(long i, long j) const { return v_[(size_t)i + (size_t)j * nr_]; }
  T &operator()(long i) { return v_[(size_t)i]; }
  const T &operator()(long i) const { return v_[(size_t)i]; }

  StridedView<T> row(long i) { return StridedView<T>{v_.data() + i, nc_, nr_}; }
  StridedView<T> col(long j) { return StridedView<T>{v_.data() + (size_t)j * nr_, nr_, 1}; }

  void setZero() {
    for (auto &x : v_) x = T(0);
  }
  Matrix &operator+=(const StridedView<T> &o) {
    for (long i = 0; i < size(); ++i) v_[(size_t)i] += o.base[i * o.stride];
    return *this;
  }

 private:
  long nr_, nc_;
  std::vector<T> v_;
};

template <typename T>
template <int R2, int C2>
StridedView<T> &StridedView<T>::operator+=(const Matrix<T, R2, C2> &o) {
  for (long i = 0; i < n; ++i) base[i * stride] += o.data()[i];
  return *this;
}

template <typename Type, int Size> using Vector = Matrix<Type, Size, 1>;

// Dense product, column-major, accumulating down each column of A so that the
// innermost loop is unit-stride.
template <typename T, int R1, int C1, int R2, int C2>
Matrix<T, R1, C2> operator*(const Matrix<T, R1, C1> &A, const Matrix<T, R2, C2> &B) {
  const long m = A.rows(), kk = A.cols(), n = B.cols();
  Matrix<T, R1, C2> out(m, n);
  T *o = out.data();
  const T *a = A.data();
  const T *b = B.data();
#pragma omp parallel for if (m * n * kk > 100000)
  for (long j = 0; j < n; ++j) {
    T *oc = o + (size_t)j * m;
    for (long p = 0; p < kk; ++p) {
      const T bpj = b[(size_t)p + (size_t)j * kk];
      const T *ac = a + (size_t)p * m;
      for (long i = 0; i < m; ++i) oc[i] += ac[i] * bpj;
    }
  }
  return out;
}

}  // namespace Eigen
