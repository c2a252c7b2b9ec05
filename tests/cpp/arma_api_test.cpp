// Unit tests of the Armadillo API subset (oracle/arma_api/armadillo) that the
// reference's CPU code is compiled against, on hand-computed values: each
// check states what Armadillo's documentation specifies for the call.
// Prints "ok N" and exits 0 when every check holds; otherwise prints the
// failing line and exits 1.
#include <armadillo>

#include <cstdio>
#include <stdexcept>
#include <vector>

static int checks = 0;
#define CHECK(cond)                                               \
  do {                                                            \
    ++checks;                                                     \
    if (!(cond)) {                                                \
      std::printf("FAILED line %d: %s\n", __LINE__, #cond);       \
      return 1;                                                   \
    }                                                             \
  } while (0)

template <class M> static bool equal(const M &a, std::vector<arma::uword> v) {
  if (a.n_elem != v.size()) return false;
  for (arma::uword i = 0; i < a.n_elem; i++)
    if (a[i] != v[i]) return false;
  return true;
}

template <class F> static bool throws_logic(F f) {
  try {
    f();
  } catch (const std::logic_error &) {
    return true;
  }
  return false;
}

int main() {
  using arma::uvec;
  using arma::umat;
  using arma::uword;

  // default shapes, sized constructors zero their elements
  uvec c0;
  CHECK(c0.n_rows == 0 && c0.n_cols == 1 && c0.n_elem == 0);
  arma::Row<uword> r0;
  CHECK(r0.n_rows == 1 && r0.n_cols == 0);
  umat m0;
  CHECK(m0.n_rows == 0 && m0.n_cols == 0);
  umat z(3, 2);
  CHECK(equal(z, {0, 0, 0, 0, 0, 0}));
  uvec z40(40);  // beyond the in-object storage
  CHECK(z40.n_elem == 40 && arma::sum(z40) == 0);
  uvec one{7};   // braces: one element holding 7
  CHECK(one.n_elem == 1 && one(0) == 7);
  CHECK(equal(arma::ones<uvec>(3), {1, 1, 1}));
  CHECK(equal(arma::zeros<uvec>(arma::size(one)), {0}));
  umat o = arma::ones<umat>(arma::size(2, 3));
  CHECK(o.n_rows == 2 && o.n_cols == 3 && arma::sum(o) == 6);

  // element access is column-major; checked accessors throw std::logic_error
  umat m(2, 3);
  for (uword i = 0; i < 6; i++) m[i] = i;  // [[0 2 4] [1 3 5]]
  CHECK(m(1, 0) == 1 && m(0, 2) == 4 && m(5) == 5);
  CHECK(throws_logic([&] { (void)m(2, 0); }));
  CHECK(throws_logic([&] { (void)m.col(3); }));
  CHECK(throws_logic([&] { (void)m.row(2); }));
  const umat &cm = m;
  CHECK(throws_logic([&] { (void)cm.col(3); }));

  // col/row: copies that read, references that write
  CHECK(equal(cm.col(1), {2, 3}));
  CHECK(equal(cm.row(1), {1, 3, 5}));
  m.col(0) = uvec{10, 11};
  CHECK(m(0, 0) == 10 && m(1, 0) == 11);
  m.row(0) = cm.row(1);
  CHECK(m(0, 0) == 11 && m(0, 1) == 3 && m(0, 2) == 5);
  CHECK(throws_logic([&] { m.col(0) = uvec{1, 2, 3}; }));

  // rows / cols / indexing by an index vector
  umat n(3, 2);
  for (uword i = 0; i < 6; i++) n[i] = 10 + i;  // cols (10 11 12) (13 14 15)
  CHECK(equal(n.rows(uvec{2, 0}), {12, 10, 15, 13}));
  CHECK(equal(n.rows(1, 2), {11, 12, 14, 15}));
  CHECK(equal(n.cols(uvec{1}), {13, 14, 15}));
  uvec v{5, 6, 7, 8};
  CHECK(equal(v(uvec{3, 0}), {8, 5}));
  CHECK(equal(v.rows(1, 2), {6, 7}));
  CHECK(throws_logic([&] { (void)v.rows(2, 4); }));

  // shed_rows by index list (any order) and by range; insert_rows adds zeros
  uvec w{1, 2, 3, 4, 5};
  w.shed_rows(uvec{3, 0});
  CHECK(equal(w, {2, 3, 5}));
  w.shed_rows(1, 2);
  CHECK(equal(w, {2}));
  uvec x{1, 2, 3};
  x.insert_rows(1, 2);
  CHECK(equal(x, {1, 0, 0, 2, 3}));
  x.insert_rows(5, 1);
  CHECK(equal(x, {1, 0, 0, 2, 3, 0}));
  umat p(2, 2);
  for (uword i = 0; i < 4; i++) p[i] = i + 1;  // [[1 3] [2 4]]
  p.insert_rows(0, 1);
  CHECK(p.n_rows == 3 && equal(p, {0, 1, 2, 0, 3, 4}));
  p.shed_rows(uvec{1});
  CHECK(equal(p, {0, 2, 0, 4}));
  umat e0(0, 3);
  e0.insert_rows(0, 1);  // a 0 x n matrix gains a zero row
  CHECK(e0.n_rows == 1 && e0.n_cols == 3 && arma::sum(e0) == 0);

  // joins: an empty operand is skipped; shapes must otherwise agree
  umat j = arma::join_horiz(umat(), uvec{1, 2});
  CHECK(j.n_rows == 2 && j.n_cols == 1);
  j = arma::join_horiz(j, uvec{3, 4});
  CHECK(equal(j, {1, 2, 3, 4}) && j.n_cols == 2);
  uvec jv = arma::join_vert(uvec(), uvec{9});
  CHECK(equal(jv, {9}));
  CHECK(equal(arma::join_vert(uvec{1, 2}, uvec{3}), {1, 2, 3}));
  CHECK(throws_logic([&] { (void)arma::join_horiz(uvec{1, 2}, uvec{3}); }));

  // repmat, transposes, vectorise, conv_to
  umat rp = arma::repmat(uvec{1, 2}, 1, 3);
  CHECK(rp.n_rows == 2 && rp.n_cols == 3 && equal(rp, {1, 2, 1, 2, 1, 2}));
  umat q(2, 3);
  for (uword i = 0; i < 6; i++) q[i] = i;
  umat qt = q.t();
  CHECK(qt.n_rows == 3 && qt.n_cols == 2 && equal(qt, {0, 2, 4, 1, 3, 5}));
  arma::Row<uword> rt = uvec{4, 5}.t();
  CHECK(rt.n_rows == 1 && rt.n_cols == 2);
  CHECK(equal(arma::vectorise(q), {0, 1, 2, 3, 4, 5}));
  std::vector<uword> sv = arma::conv_to<std::vector<uword>>::from(arma::vectorise(qt));
  CHECK(sv.size() == 6 && sv[1] == 2 && sv[3] == 1);

  // reductions: sum of everything; prod of a vector, or per column of a matrix
  CHECK(arma::sum(uvec{1, 2, 3}) == 6);
  CHECK(arma::prod(uvec{2, 3, 4}) == 24);
  CHECK(arma::prod(uvec()) == 1);
  arma::Row<uword> pc = arma::prod(q + arma::ones<umat>(arma::size(q)));  // (1*2, 3*4, 5*6)
  CHECK(equal(pc, {2, 12, 30}) && arma::sum(pc) == 44);
  CHECK(equal(pc.t(), {2, 12, 30}));

  // elementwise arithmetic and relations, min/max of two vectors
  uvec a{1, 5, 3}, b{2, 2, 3};
  CHECK(equal(a + b, {3, 7, 6}));
  CHECK(equal(a - uvec{1, 1, 1}, {0, 4, 2}));
  CHECK(equal(a % b, {2, 10, 9}));
  CHECK(equal(a >= b, {0, 1, 1}));
  CHECK(equal(a <= b, {1, 0, 1}));
  CHECK(equal(a == b, {0, 0, 1}));
  CHECK(equal(arma::max(a, b), {2, 5, 3}));
  CHECK(equal(arma::min(a, b), {1, 2, 3}));
  CHECK(arma::all(a >= uvec{1, 1, 1}) && !arma::all(a >= b));
  CHECK(arma::any(a > b) && !arma::any(a > uvec{9, 9, 9}));
  CHECK(throws_logic([&] { (void)(a + uvec{1, 2}); }));
  arma::Col<int> flags{0, 3, 0, -1};
  CHECK(equal(arma::find(flags), {1, 3}));
  CHECK(equal(arma::find(flags != 0), {1, 3}));

  // sort_index: ascending, equal keys keep their order; is_sorted: non-descending
  CHECK(equal(arma::sort_index(uvec{3, 1, 2}), {1, 2, 0}));
  CHECK(equal(arma::sort_index(uvec{1, 1, 1, 0}), {3, 0, 1, 2}));
  CHECK(uvec({1, 1, 2}).is_sorted() && !uvec({2, 1}).is_sorted());

  // matrix product (the loop: no BLAS registered here)
  arma::mat A(2, 3), B(3, 2);
  for (uword i = 0; i < 6; i++) A[i] = double(i + 1);   // [[1 3 5] [2 4 6]]
  for (uword i = 0; i < 6; i++) B[i] = double(i + 7);   // [[7 10] [8 11] [9 12]]
  arma::mat C = A * B;  // [[76 103] [100 136]]
  CHECK(C.n_rows == 2 && C.n_cols == 2);
  CHECK(C(0, 0) == 76.0 && C(1, 0) == 100.0 && C(0, 1) == 103.0 && C(1, 1) == 136.0);
  CHECK(throws_logic([&] { (void)(A * A); }));

  // initializer lists: a flat list is one row, a list of lists gives the rows
  umat fr({1, 0});
  CHECK(fr.n_rows == 1 && fr.n_cols == 2 && fr(0, 0) == 1 && fr(0, 1) == 0);
  umat lr{{1, 0}, {0, 1}, {2, 3}};
  CHECK(lr.n_rows == 3 && lr.n_cols == 2 && equal(lr, {1, 0, 2, 0, 1, 3}));
  CHECK(throws_logic([&] { umat bad{{1, 2}, {3}}; }));
  arma::mat dm{{0, 1}, {2, 3}};
  CHECK(arma::accu(dm % dm.t()) == 0.0 + 2.0 + 2.0 + 9.0);
  // unique: distinct elements ascending; shed_row; a column from std::vector
  CHECK(equal(arma::unique(uvec{3, 1, 3, 2, 1}), {1, 2, 3}));
  uvec sr{4, 5, 6};
  sr.shed_row(1);
  CHECK(equal(sr, {4, 6}));
  std::vector<uword> stdv{8, 9};
  uvec fromv(stdv);
  CHECK(equal(fromv, {8, 9}));
  // a relation with a plain integer literal
  CHECK(equal(uvec{0, 2, 0} == 0, {1, 0, 1}));
  CHECK(equal(arma::find(uvec{0, 2, 0} != 0), {1}));

  // arithmetic with a scalar on the right; randu in [0, 1)
  CHECK(equal(uvec{4, 5} - 1, {3, 4}) && equal(uvec{4, 5} + 2, {6, 7}));
  CHECK(equal(uvec{4, 6} * 2, {8, 12}) && equal(uvec{4, 6} / 2, {2, 3}));
  arma::vec r = arma::randu<arma::vec>(100);
  CHECK(r.n_rows == 100 && r.n_cols == 1);
  bool in_range = true;
  for (uword i = 0; i < r.n_elem; i++) in_range = in_range && r[i] >= 0.0 && r[i] < 1.0;
  const double u1 = arma::randu();
  CHECK(in_range && u1 >= 0.0 && u1 < 1.0 && r[0] != r[1]);

  // copies of large (heap) and small (in-object) vectors are independent
  uvec big(20);
  big[19] = 5;
  uvec big2 = big;
  big2[19] = 6;
  CHECK(big[19] == 5 && big2[19] == 6);
  uvec moved = std::move(big2);
  CHECK(moved[19] == 6);
  uvec small{1, 2};
  uvec small2 = small;
  small2[0] = 9;
  CHECK(small[0] == 1);

  std::printf("ok %d\n", checks);
  return 0;
}
