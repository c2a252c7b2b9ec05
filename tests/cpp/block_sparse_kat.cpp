// The reference's known answers (test/gpu/block_sparse_test.cu:10-231) run
// through the C++ drop-in class torque::gpu::BlockSparseTensor<T>, written the
// way a reference user writes them, for T = float, double and half (the
// reference's instantiations, src/gpu/block_sparse.cu:66-148).  Exit status = number of failed checks.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "torque_gb300/block_sparse.hpp"

static int g_failed = 0;
#define EXPECT(cond)                                                   \
  do {                                                                 \
    if (!(cond)) {                                                     \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);    \
      g_failed++;                                                      \
    }                                                                  \
  } while (0)

// values compared as float or double (binary16 has no built-in comparison on the host)
static float val(float x) { return x; }
static double val(double x) { return x; }
static float val(__half x) { return __half2float(x); }

template <typename T>
void run_cases() {
  using torque::gpu::BlockSparseTensor;
  int handle = 0;  // stands in for the cuBLAS handle the reference passes

  {  // matrix: init, query, modify, append
    std::vector<T> a = {1, 2, 3, 4};
    BlockSparseTensor<T> t(a.data(), arma::uvec{1, 1}, arma::uvec{2, 2}, arma::uvec{4, 3});
    EXPECT(val(t.query({1, 1})) == 1);
    EXPECT(val(t.query({2, 2})) == 4);
    EXPECT(val(t.query({3, 2})) == 0);
    t.modify({2, 2}, 0);
    EXPECT(val(t.query({2, 2})) == 0);
    t.modify({3, 2}, 5);
    EXPECT(val(t.query({3, 2})) == 5);
    t.append_block(a.data(), {0, 0}, {1, 1}, {1, 2});
    EXPECT(val(t.query({1, 1})) == 5);
    EXPECT(t.block_offsets.n_elem == 3);
  }
  {  // matrix transposition
    std::vector<T> a = {1, 2, 3, 4};
    BlockSparseTensor<T> t(a.data(), arma::uvec{2, 0}, arma::uvec{3, 1}, arma::uvec{4, 3});
    t = t.hard_transpose({1, 0});
    EXPECT(val(t.query({0, 3})) == 2);
    EXPECT(val(t.query({1, 2})) == 3);
    const auto back = t.hard_transpose({1, 0});
    EXPECT(val(back.query({3, 0})) == 2);
    EXPECT(val(back.query({2, 1})) == 3);
  }
  {  // rank-3 tensor: empty, then one appended block
    BlockSparseTensor<T> t(arma::uvec{2, 2, 3});
    EXPECT(val(t.query({1, 1, 0})) == 0);
    std::vector<T> a = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12};
    t.append_block(a.data(), {0, 0, 0}, {1, 1, 2}, {1, 2, 4});
    EXPECT(val(t.query({0, 1, 2})) == 11);
  }
  {  // rank-3 transposition with overlapping blocks
    std::vector<T> a = {1, 2, 3, 4, 5, 6, 0, 0, 0, 0, 0, 0};
    std::vector<T> b = {7, 8, 9, 10, 11, 12};
    BlockSparseTensor<T> t(arma::uvec{2, 2, 3});
    t.append_block(a.data(), {0, 0, 0}, {1, 1, 2}, {1, 2, 4});
    t.append_block(b.data(), {1, 0, 0}, {1, 1, 2}, {1, 1, 2});
    const auto p = t.hard_transpose({1, 0, 2});
    EXPECT(val(p.query({1, 0, 0})) == 3);
    EXPECT(val(p.query({1, 0, 1})) == 0);
    EXPECT(val(p.query({1, 1, 2})) == 12);
  }
  {  // scalar
    BlockSparseTensor<T> t(arma::uvec{});
    EXPECT(t.rank == 0);
    EXPECT(val(t.query({})) == 0);
    t.modify({}, 1);
    EXPECT(val(t.query({})) == 1);
  }
  {  // vector with itself -> 30
    std::vector<T> v1{0, 1}, v2{2, 3, 4};
    BlockSparseTensor<T> t(arma::uvec{5});
    t.append_block(v1.data(), {0}, {1}, {1});
    t.append_block(v2.data(), {2}, {4}, {1});
    EXPECT(val(t.contract(handle, t, arma::umat({{0, 0}})).to_number()) == 30);
  }
  {  // block-diagonal matrix squared
    std::vector<T> b1{0, 1, 2, 3}, b2{4, 5, 6, 7};
    BlockSparseTensor<T> t(arma::uvec{4, 4});
    t.append_block(b1.data(), {0, 0}, {1, 1}, {1, 2});
    t.append_block(b2.data(), {2, 2}, {3, 3}, {1, 2});
    const auto sq = t.contract(handle, t, arma::umat({1, 0}));
    const T want[4][4] = {{2, 6, 0, 0}, {3, 11, 0, 0}, {0, 0, 46, 66}, {0, 0, 55, 79}};
    for (arma::uword i = 0; i < 4; i++)
      for (arma::uword j = 0; j < 4; j++) EXPECT(val(sq.query({i, j})) == val(want[i][j]));
  }
  {  // matrix inner product over both legs -> 206
    std::vector<T> b1{0, 1, 2, 3}, b2{0, 7, 8, 9};
    BlockSparseTensor<T> t(arma::uvec{3, 3});
    t.append_block(b1.data(), {0, 0}, {1, 1}, {1, 2});
    t.append_block(b2.data(), {1, 1}, {2, 2}, {1, 2});
    EXPECT(val(t.contract(handle, t, arma::umat{{1, 0}, {0, 1}}).to_number()) == 206);
  }
  {  // tensor-vector over each leg
    std::vector<T> d1{0, 1, 2, 3}, d2{4, 5, 6, 7}, v{1, 2};
    BlockSparseTensor<T> t(arma::uvec{2, 2, 2});
    t.append_block(d1.data(), {0, 0, 0}, {1, 1, 0}, {1, 2, 4});
    t.append_block(d2.data(), {0, 0, 1}, {1, 1, 1}, {1, 2, 4});
    BlockSparseTensor<T> vec(arma::uvec{2});
    vec.append_block(v.data(), {0}, {1}, {1});
    const auto c0 = t.contract(handle, vec, arma::umat{{0, 0}});
    EXPECT(val(c0.query({0, 0})) == 2 && val(c0.query({1, 0})) == 8);
    EXPECT(val(c0.query({0, 1})) == 14 && val(c0.query({1, 1})) == 20);
    const auto c1 = t.contract(handle, vec, arma::umat{{1, 0}});
    EXPECT(val(c1.query({0, 0})) == 4 && val(c1.query({1, 0})) == 7);
    EXPECT(val(c1.query({0, 1})) == 16 && val(c1.query({1, 1})) == 19);
    const auto c2 = t.contract(handle, vec, arma::umat{{2, 0}});
    EXPECT(val(c2.query({1, 0})) == 11);
  }
  {  // tensor-matrix over two legs, blocks appended in reverse
    std::vector<T> d1{0, 1, 2, 3}, d2{4, 5, 6, 7}, d3{8, 9, 10, 11}, m{1, 2, 3, 4};
    BlockSparseTensor<T> t(arma::uvec{2, 2, 3});
    t.append_block(d3.data(), {0, 0, 2}, {1, 1, 2}, {1, 2, 4});
    t.append_block(d2.data(), {0, 0, 1}, {1, 1, 1}, {1, 2, 4});
    t.append_block(d1.data(), {0, 0, 0}, {1, 1, 0}, {1, 2, 4});
    BlockSparseTensor<T> mat(arma::uvec{2, 2});
    mat.append_block(m.data(), {0, 0}, {1, 1}, {1, 2});
    const auto c = t.contract(handle, mat, arma::umat{{0, 1}, {1, 0}});
    EXPECT(val(c.query({0})) == 19 && val(c.query({1})) == 59 && val(c.query({2})) == 99);
    // the public metadata mirrors the reference's members
    EXPECT(c.rank == 1 && c.dimension(0) == 3);
    EXPECT(c.begin_points.n_cols == 3 && c.block_offsets(2) == 2);
  }
  {  // charge-conserving construction (an extension): U(1) legs q in {0, 1}
     // sized {1, 2}, legs 0 in and 1 out -> blocks (0,0) and (1,1)
    std::vector<arma::Col<long long>> q = {arma::Col<long long>{0, 1},
                                           arma::Col<long long>{0, 1}};
    std::vector<arma::uvec> sz = {arma::uvec{1, 2}, arma::uvec{1, 2}};
    std::vector<T> d = {7, 1, 2, 3, 4};
    const auto c = BlockSparseTensor<T>::from_charges(q, sz, {1, -1}, d.data());
    EXPECT(c.begin_points.n_cols == 2 && c.dimension(0) == 3);
    EXPECT(val(c.query({0, 0})) == 7 && val(c.query({1, 2})) == 3);
    EXPECT(val(c.query({0, 1})) == 0);
  }
  {  // misuse throws Error like the reference
    BlockSparseTensor<T> a(arma::uvec{4, 3}), b(arma::uvec{5, 3});
    bool thrown = false;
    try {
      a.contract(b, arma::umat{{0, 0}});
    } catch (const Error &e) {
      thrown = std::string(e.what()).find("do not match") != std::string::npos;
    }
    EXPECT(thrown);
    thrown = false;
    try {
      val(a.query({4, 0}));
    } catch (const Error &) {
      thrown = true;
    }
    EXPECT(thrown);
  }
}

// The extensions from C++: a Z2 tensor filled with set_data, its QR
// reproducing it through contract, and its singular values carrying its
// Frobenius norm.
static void factorisations() {
  using torque::gpu::BlockSparseTensor;
  std::vector<arma::Col<long long>> q = {{0, 1}, {0, 1}, {0, 1}};
  std::vector<arma::uvec> sz = {{3, 2}, {2, 4}, {3, 3}};
  auto t = BlockSparseTensor<double>::from_charges(q, sz, {1, 1, -1}, nullptr, 0, 2);
  arma::uword n = 0;
  for (arma::uword k = 0; k < t.block_n_elem.n_elem; k++) n += t.block_n_elem(k);
  std::vector<double> v(n);
  for (arma::uword i = 0; i < n; i++) v[i] = std::sin(1.0 + (double)i) + 0.25 * (double)(i % 3);
  t.set_data(v.data());
  double norm2 = 0, mx = 0;
  for (double x : v) norm2 += x * x, mx = std::max(mx, std::fabs(x));
  auto qr = t.qr(arma::uvec{0, 1});
  auto back = qr.first.contract(qr.second, arma::umat{{2, 0}});
  double worst = 0;
  for (arma::uword i = 0; i < 5; i++)
    for (arma::uword j = 0; j < 6; j++)
      for (arma::uword k = 0; k < 6; k++)
        worst = std::max(worst, std::fabs(back.query({i, j, k}) - t.query({i, j, k})));
  EXPECT(worst <= 1e-12 * mx);
  auto svd = t.svd(arma::uvec{0, 1});
  const BlockSparseTensor<double> &s = std::get<1>(svd);
  double s2 = 0;
  for (arma::uword k = 0; k < s.dimension(0); k++) s2 += s.query({k}) * s.query({k});
  EXPECT(std::fabs(s2 - norm2) <= 1e-12 * norm2);
}

// The raw move-in constructor (block_sparse.cuh:283-304): a cudaMalloc'd
// buffer holding two column-major blocks of a 4 x 3 matrix, rows 0-1 x
// columns 0-1 (values 1..4) and rows 1-3 x columns 1-2 (values 5..10), is
// adopted without a copy and read back (the blocks overlap at (1, 1): 4 + 5);
// append_block then replaces the adopted buffer (the tensor frees it) and the
// tensor's destructor frees the rest.  Metadata that disagrees with the boxes
// throws Error before anything is adopted.
static void move_in() {
  using torque::gpu::BlockSparseTensor;
  const std::vector<double> h = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10};
  double *d = nullptr;
  EXPECT(cudaMalloc(reinterpret_cast<void **>(&d), h.size() * sizeof(double)) == cudaSuccess);
  EXPECT(cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice) ==
         cudaSuccess);
  bool threw = false;
  try {  // blocks_dimension says block 1 has one column; its box has two
    BlockSparseTensor<double> bad(d, 2, arma::uvec{4, 3}, arma::umat{{2, 3}, {2, 1}},
                                  arma::umat{{0, 1}, {0, 1}}, arma::umat{{1, 3}, {1, 2}},
                                  arma::uvec{4, 6}, arma::uvec{0, 4}, arma::umat{{1, 1}, {2, 3}});
  } catch (const Error &) {
    threw = true;
  }
  EXPECT(threw);
  BlockSparseTensor<double> t(d, 2, arma::uvec{4, 3}, arma::umat{{2, 3}, {2, 2}},
                              arma::umat{{0, 1}, {0, 1}}, arma::umat{{1, 3}, {1, 2}},
                              arma::uvec{4, 6}, arma::uvec{0, 4}, arma::umat{{1, 1}, {2, 3}});
  EXPECT(t.begin_points.n_cols == 2 && t.block_offsets(1) == 4 && t.index_tables(1, 1) == 3);
  EXPECT(t.query({0, 0}) == 1 && t.query({1, 0}) == 2 && t.query({0, 1}) == 3);
  EXPECT(t.query({1, 1}) == 4 + 5);
  EXPECT(t.query({1, 2}) == 8 && t.query({3, 2}) == 10 && t.query({0, 2}) == 0);
  const std::vector<double> extra = {11};
  t.append_block(extra.data(), arma::uvec{3, 0}, arma::uvec{3, 0}, arma::uvec{1, 1});
  EXPECT(t.query({3, 0}) == 11 && t.query({3, 2}) == 10 && t.query({1, 1}) == 9);
}

int main() {
  run_cases<float>();
  run_cases<double>();
  run_cases<__half>();
  factorisations();
  move_in();
  std::printf("%s (%d failed checks)\n", g_failed ? "FAIL" : "OK", g_failed);
  return g_failed;
}
