// torque::gpu::DenseTensor<T> over the C ABI of libtorque_gb300.
//
// The reference class (src/gpu/dense.cuh:52-604) keeps one thrust vector and
// contracts through cuTT + one cuBLAS GEMM (or cuTENSOR).  Here a dense tensor
// is a block-sparse tensor with a single block spanning the whole box, so
// contract and hard_transpose run the library's own grouped GEMM and
// transpose kernels.  Same constructors, members and errors as the reference;
// contract() takes the reference's handle argument and ignores it, and accepts
// tq_contract_opts for the tensor-core forms.
#pragma once

#include "block_sparse.hpp"

namespace torque {
namespace gpu {

namespace detail {
// Column-major strides of a dense box (torque::util::generate_index_table,
// src/util/space.h:11-24).
inline arma::uvec index_table_of(const arma::uvec &dim) {
  arma::uvec t(dim.n_elem);
  arma::uword s = 1;
  for (arma::uword l = 0; l < dim.n_elem; l++) {
    t(l) = s;
    s *= dim(l);
  }
  return t;
}

inline arma::uvec permuted(const arma::uvec &v, const arma::uvec &perm) {
  arma::uvec out(perm.n_elem);
  for (arma::uword l = 0; l < perm.n_elem; l++) out(l) = v(perm(l));
  return out;
}

inline void shape_of(tq_bs *h, arma::uword &rank, arma::uvec &dimension) {
  tq_dtype dt;
  int32_t r = 0;
  int64_t nb = 0, ne = 0;
  check(tq_bs_shape(h, &dt, &r, &nb, &ne));
  std::vector<int64_t> d(r);
  check(tq_bs_metadata(h, r ? d.data() : nullptr, nullptr, nullptr, nullptr, nullptr));
  rank = (arma::uword)r;
  dimension = arma::uvec((arma::uword)r);
  for (int32_t l = 0; l < r; l++) dimension(l) = (arma::uword)d[l];
}

inline void contract_legs(const arma::umat &ci, std::vector<int64_t> &al,
                          std::vector<int64_t> &bl) {
  al.resize(ci.n_rows);
  bl.resize(ci.n_rows);
  for (arma::uword k = 0; k < ci.n_rows; k++) {
    al[k] = (int64_t)ci(k, 0);
    bl[k] = (int64_t)ci(k, 1);
  }
}
}  // namespace detail

template <typename T>
class DenseTensor {
 public:
  arma::uword rank = 0;
  arma::uvec dimension;
  arma::uvec index_table;

  // DenseTensor(dimension) (dense.cuh:68-84): all zeros.
  explicit DenseTensor(const arma::uvec &dim) { make(dim, nullptr); }

  // DenseTensor(source, dimension) (dense.cuh:86-114): host data, column-major.
  explicit DenseTensor(const T *source_data, const arma::uvec &dim) {
    if (!source_data) throw Error("Source data not allocated!");
    make(dim, source_data);
  }

  DenseTensor(const DenseTensor &o)
      : rank(o.rank), dimension(o.dimension), index_table(o.index_table) {
    detail::check(tq_bs_clone(o.h_, nullptr, &h_));
  }
  DenseTensor(DenseTensor &&o) noexcept
      : rank(o.rank), dimension(std::move(o.dimension)), index_table(std::move(o.index_table)) {
    std::swap(h_, o.h_);
  }
  DenseTensor &operator=(DenseTensor &&o) noexcept {
    rank = o.rank;
    dimension = std::move(o.dimension);
    index_table = std::move(o.index_table);
    std::swap(h_, o.h_);
    return *this;
  }
  DenseTensor &operator=(const DenseTensor &o) {
    if (this != &o) {
      DenseTensor c(o);
      *this = std::move(c);
    }
    return *this;
  }
  ~DenseTensor() {
    if (h_) tq_bs_destroy(h_);
  }

  T to_number() const {
    T v = T(0);
    detail::check(tq_bs_to_number(h_, &v));
    return v;
  }

  // initialize(source) (dense.cuh:172-184): overwrite every element.
  void initialize(const T *source_data) {
    if (!source_data) throw Error("Source data not allocated!");
    detail::check(tq_bs_set_data(h_, source_data, TQ_MEM_HOST, nullptr));
  }

  void modify(const arma::uvec &indices, const T number) {
    check_indices(indices);
    const auto idx = detail::flat(indices);
    detail::check(tq_bs_modify(h_, rank ? idx.data() : nullptr, &number));
  }

  T query(const arma::uvec &indices) const {
    check_indices(indices);
    const auto idx = detail::flat(indices);
    T v = T(0);
    detail::check(tq_bs_query(h_, rank ? idx.data() : nullptr, &v));
    return v;
  }

  // contract(handle, tensor, contracting_indices) (dense.cuh:439-555).
  template <typename Handle>
  DenseTensor contract(Handle, const DenseTensor &tensor, const arma::umat &contracting_indices,
                       const tq_contract_opts *opts = nullptr) const {
    return contract(tensor, contracting_indices, opts);
  }
  DenseTensor contract(const DenseTensor &tensor, const arma::umat &contracting_indices,
                       const tq_contract_opts *opts = nullptr) const {
    std::vector<int64_t> al, bl;
    detail::contract_legs(contracting_indices, al, bl);
    tq_bs *out = nullptr;
    detail::check(tq_bs_contract(h_, tensor.h_, (int32_t)al.size(), al.data(), bl.data(), opts,
                                 nullptr, &out));
    return DenseTensor(out);
  }

  // hard_transpose(permutation) (dense.cuh:561-599).
  DenseTensor hard_transpose(const arma::uvec &permutation) const {
    if (permutation.n_elem != rank)
      throw Error("The number of permutation does not match the rank of tensor");
    const auto p = detail::flat(permutation);
    tq_bs *out = nullptr;
    detail::check(tq_bs_hard_transpose(h_, p.data(), nullptr, &out));
    return DenseTensor(out);
  }

  tq_bs *handle() const { return h_; }

 private:
  explicit DenseTensor(tq_bs *h) : h_(h) {
    detail::shape_of(h_, rank, dimension);
    index_table = detail::index_table_of(dimension);
  }

  void make(const arma::uvec &dim, const T *src) {
    rank = dim.n_elem;
    dimension = dim;
    index_table = detail::index_table_of(dim);
    const auto d = detail::flat(dim);
    if (rank == 0) {
      if (src)
        detail::check(tq_bs_create(detail::dtype<T>(), 0, nullptr, 0, nullptr, nullptr, nullptr,
                                   src, TQ_MEM_HOST, nullptr, &h_));
      else
        detail::check(tq_bs_create_empty(detail::dtype<T>(), 0, nullptr, &h_));
      return;
    }
    std::vector<int64_t> b(rank, 0), e(rank);
    for (arma::uword l = 0; l < rank; l++) e[l] = d[l] - 1;
    if (src)
      detail::check(tq_bs_create(detail::dtype<T>(), (int32_t)rank, d.data(), 1, b.data(),
                                 e.data(), nullptr, src, TQ_MEM_HOST, nullptr, &h_));
    else
      detail::check(tq_bs_create_zeros(detail::dtype<T>(), (int32_t)rank, d.data(), 1, b.data(),
                                       e.data(), nullptr, nullptr, &h_));
  }

  void check_indices(const arma::uvec &indices) const {
    if (indices.n_elem != rank) throw Error("Rank does not match");
    for (arma::uword l = 0; l < rank; l++)
      if (indices(l) >= dimension(l)) throw Error("Indices out of boundary");
  }

  tq_bs *h_ = nullptr;
};

}  // namespace gpu
}  // namespace torque
