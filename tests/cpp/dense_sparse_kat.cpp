// The reference's known answers for its dense and element-sparse GPU classes
// (test/gpu/dense_test.cu:7-300, test/gpu/sparse_test.cu:31-319) run through
// torque::gpu::DenseTensor<T> and SparseTensor<T> over libtorque_gb300,
// written the way a reference user writes them.  Exit status = failed checks.
#include <cstdio>
#include <vector>

#include "torque_gb300/sparse.hpp"

static int g_failed = 0;
#define EXPECT(cond)                                                   \
  do {                                                                 \
    if (!(cond)) {                                                     \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);    \
      g_failed++;                                                      \
    }                                                                  \
  } while (0)

static arma::uvec table(const arma::uvec &d) { return torque::gpu::detail::index_table_of(d); }

template <typename T>
void dense_cases() {
  using torque::gpu::DenseTensor;
  int handle = 0;  // stands in for the cuBLAS handle the reference passes
  std::vector<T> a = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12};
  {
    DenseTensor<T> t(arma::uvec{4, 3});
    EXPECT(t.query({1, 1}) == 0);
    t.initialize(a.data());
    EXPECT(t.query({1, 2}) == 10);
    t = t.hard_transpose({1, 0});
    EXPECT(t.query({1, 2}) == 7);
    const auto back = t.hard_transpose({1, 0});
    for (arma::uword i = 0; i < 3; i++)
      for (arma::uword j = 0; j < 4; j++) EXPECT(t.query(arma::uvec{i, j}) == back.query(arma::uvec{j, i}));
  }
  {
    DenseTensor<T> t(a.data(), arma::uvec{2, 2, 3});
    EXPECT(t.query({0, 0, 2}) == 9);
    EXPECT(t.query({0, 1, 2}) == 11);
    t = t.hard_transpose({0, 2, 1});
    EXPECT(t.query({0, 2, 0}) == 9);
    EXPECT(t.query({0, 2, 1}) == 11);
  }
  {
    DenseTensor<T> s(arma::uvec{});
    EXPECT(s.rank == 0);
    EXPECT(s.query({}) == 0);
    s.modify({}, 1);
    EXPECT(s.query({}) == 1);
  }
  {
    std::vector<T> v = {0, 1, 2, 3, 4};
    const DenseTensor<T> t(v.data(), arma::uvec{5});
    EXPECT(t.contract(handle, t, arma::umat({0, 0})).to_number() == 30);
  }
  {
    std::vector<T> v = {0, 1, 2, 3, 4, 5, 6, 7, 8};
    const DenseTensor<T> t(v.data(), arma::uvec{3, 3});
    const auto sq = t.contract(handle, t, arma::umat({1, 0}));
    const T ref[3][3] = {{15, 42, 69}, {18, 54, 90}, {21, 66, 111}};
    for (arma::uword i = 0; i < 3; i++)
      for (arma::uword j = 0; j < 3; j++) EXPECT(sq.query(arma::uvec{i, j}) == ref[i][j]);
    EXPECT(t.contract(handle, t, arma::umat({{1, 0}, {0, 1}})).to_number() == 180);
  }
  {
    std::vector<T> td = {0, 1, 2, 3, 4, 5, 6, 7}, vd = {1, 2};
    const DenseTensor<T> t(td.data(), arma::uvec{2, 2, 2});
    const DenseTensor<T> v(vd.data(), arma::uvec{2});
    const auto c = t.contract(handle, v, arma::umat{{0, 0}});
    EXPECT(c.query({0, 0}) == 2);
    EXPECT(c.query({1, 0}) == 8);
    EXPECT(c.query({0, 1}) == 14);
    EXPECT(c.query({1, 1}) == 20);
    EXPECT(t.contract(handle, v, arma::umat{{2, 0}}).query({1, 0}) == 11);
  }
  {
    std::vector<T> td = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11}, md = {1, 2, 3, 4};
    const DenseTensor<T> t(td.data(), arma::uvec{2, 2, 3});
    const DenseTensor<T> m(md.data(), arma::uvec{2, 2});
    const auto c = t.contract(handle, m, arma::umat{{0, 1}, {1, 0}});
    EXPECT(c.query({0}) == 19);
    EXPECT(c.query({1}) == 59);
    EXPECT(c.query({2}) == 99);
  }
}

template <typename T>
void sparse_cases() {
  using torque::gpu::SparseTensor;
  int handle = 0;
  std::vector<T> a = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12};
  const arma::uvec idx12 = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
  {
    SparseTensor<T> t(arma::uvec{4, 3});
    EXPECT(t.query({1, 1}) == 0);
    t.initialize(a.data(), idx12);
    EXPECT(t.query({1, 2}) == 10);
    t.soft_transpose({1, 0});
    EXPECT(t.query({1, 2}) == 7);
    const auto back = t.hard_transpose({1, 0});
    for (arma::uword i = 0; i < 3; i++)
      for (arma::uword j = 0; j < 4; j++) EXPECT(t.query(arma::uvec{i, j}) == back.query(arma::uvec{j, i}));
  }
  {
    const arma::uvec dim = {2, 2, 3};
    SparseTensor<T> t(a.data(), idx12, table(dim), dim);
    EXPECT(t.query({0, 0, 2}) == 9);
    EXPECT(t.query({0, 1, 2}) == 11);
    t.soft_transpose({0, 2, 1});
    EXPECT(t.query({0, 2, 0}) == 9);
    EXPECT(t.query({0, 2, 1}) == 11);
    const auto u = t.hard_transpose({1, 0, 2});
    EXPECT(u.query({2, 0, 0}) == 9);
    EXPECT(u.query({2, 0, 1}) == 11);
  }
  {
    SparseTensor<T> s(arma::uvec{});
    EXPECT(s.rank == 0);
    EXPECT(s.query({}) == 0);
    s.modify({}, 1);
    EXPECT(s.query({}) == 1);
  }
  {
    std::vector<T> v = {0, 1, 2, 3, 4};
    const arma::uvec dim = {5};
    const SparseTensor<T> t(v.data(), arma::uvec{0, 1, 2, 3, 4}, table(dim), dim);
    EXPECT(t.contract(handle, t, arma::umat({0, 0})).to_number() == 30);
  }
  {
    std::vector<T> v = {0, 1, 2, 3, 4, 5, 6, 7, 8};
    const arma::uvec dim = {3, 3};
    const SparseTensor<T> t(v.data(), arma::uvec{0, 1, 2, 3, 4, 5, 6, 7, 8}, table(dim), dim);
    const auto sq = t.contract(handle, t, arma::umat({1, 0}));
    const T ref[3][3] = {{15, 42, 69}, {18, 54, 90}, {21, 66, 111}};
    for (arma::uword i = 0; i < 3; i++)
      for (arma::uword j = 0; j < 3; j++) EXPECT(sq.query(arma::uvec{i, j}) == ref[i][j]);
    EXPECT(t.contract(handle, t, arma::umat({{1, 0}, {0, 1}})).to_number() == 180);
  }
  {
    std::vector<T> td = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11}, md = {1, 2, 3, 4};
    const arma::uvec dt = {2, 2, 3}, dm = {2, 2};
    const SparseTensor<T> t(td.data(), idx12, table(dt), dt);
    const SparseTensor<T> m(md.data(), arma::uvec{0, 1, 2, 3}, table(dm), dm);
    const auto c = t.contract(handle, m, arma::umat{{0, 1}, {1, 0}});
    EXPECT(c.query({0}) == 19);
    EXPECT(c.query({1}) == 59);
    EXPECT(c.query({2}) == 99);
    EXPECT(c.indices.size() == 3);
  }
}

int main() {
  dense_cases<float>();
  dense_cases<double>();
  sparse_cases<float>();
  sparse_cases<double>();
  if (g_failed == 0) std::printf("OK\n");
  return g_failed;
}
