// Minimal stand-in for the parts of Armadillo's API that appear in the
// signatures of torque::gpu::BlockSparseTensor: arma::uword, Mat<T>/umat and
// Col<T>/uvec (a column is a one-column matrix, so a uvec binds to a
// const umat&), column-major, constructed from initializer lists the way
// Armadillo documents (a nested list gives the rows, a flat list one row for a
// matrix and one column for a column vector).  Used only when the real
// <armadillo> header is not available; the memory layout (memptr,
// column-major) is the same, so the C ABI receives identical arrays either way.
#pragma once
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <vector>

namespace arma {

using uword = unsigned long long;

template <typename T>
class Mat {
 public:
  Mat() = default;
  Mat(uword r, uword c) { resize(r, c); }
  Mat(std::initializer_list<std::initializer_list<T>> rows) {
    resize(rows.size(), rows.size() ? rows.begin()->size() : 0);
    uword r = 0;
    for (const auto &row : rows) {
      if (row.size() != n_cols) throw std::logic_error("Mat(): rows of different length");
      uword c = 0;
      for (const T &x : row) v_[r + c++ * n_rows] = x;
      ++r;
    }
  }
  Mat(std::initializer_list<T> row) {
    resize(1, row.size());
    uword c = 0;
    for (const T &x : row) v_[c++] = x;
  }
  T &operator()(uword r, uword c) { return v_[index(r, c)]; }
  const T &operator()(uword r, uword c) const { return v_[index(r, c)]; }
  T *memptr() { return v_.data(); }
  const T *memptr() const { return v_.data(); }
  bool is_empty() const { return n_elem == 0; }
  uword n_rows = 0, n_cols = 0, n_elem = 0;

 protected:
  void resize(uword r, uword c) {
    n_rows = r;
    n_cols = c;
    n_elem = r * c;
    v_.assign(n_elem, T(0));
  }
  uword index(uword r, uword c) const {
    if (r >= n_rows || c >= n_cols) throw std::out_of_range("Mat::operator(): index out of bounds");
    return r + c * n_rows;
  }
  std::vector<T> v_;
};

template <typename T>
class Col : public Mat<T> {
 public:
  Col() { this->resize(0, 1); }
  explicit Col(uword n) { this->resize(n, 1); }
  Col(std::initializer_list<T> l) {
    this->resize(l.size(), 1);
    uword i = 0;
    for (const T &x : l) this->v_[i++] = x;
  }
  T &operator()(uword i) { return this->v_[at(i)]; }
  const T &operator()(uword i) const { return this->v_[at(i)]; }
  T &operator[](uword i) { return this->v_[i]; }
  const T &operator[](uword i) const { return this->v_[i]; }

 private:
  uword at(uword i) const {
    if (i >= this->n_elem) throw std::out_of_range("Col::operator(): index out of bounds");
    return i;
  }
};

using uvec = Col<uword>;
using umat = Mat<uword>;
using vec = Col<double>;
using mat = Mat<double>;

}  // namespace arma
