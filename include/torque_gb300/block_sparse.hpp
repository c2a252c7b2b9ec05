// torque::gpu::BlockSparseTensor<T> over the C ABI of libtorque_gb300.
//
// Source-compatible with the reference class (src/gpu/block_sparse.cuh:143-1181):
// the same constructors, public metadata members, element access, contract,
// hard_transpose and slice, with T in {float, double, half}.  Differences:
//   * contract() takes any handle type in the first position and ignores it (no
//     cuBLAS is used); an overload without a handle is added;
//   * API misuse throws Error (as the reference does); CUDA failures throw
//     std::runtime_error instead of exiting the process;
//   * contract() accepts a tq_contract_opts for the tensor-core forms and the
//     reduced layout.
// The public members are refreshed from the library after every call that
// changes the block list.
#pragma once

#if __has_include(<armadillo>) && !defined(TORQUE_GB300_NO_ARMADILLO)
#include <armadillo>
#else
#include "arma_min.hpp"
#endif

#include <cuda_runtime_api.h>

#include <stdexcept>
#include <string>
#include <type_traits>

#include <cuda_fp16.h>
#include <tuple>
#include <utility>
#include <vector>

#include "../torque_gb300.h"

#ifndef TORQUE_ERROR_H
struct Error : public std::runtime_error {
  explicit Error(const std::string &error_message)
      : std::runtime_error("Error: " + error_message) {}
  explicit Error(const char *error_message)
      : std::runtime_error("Error: " + std::string(error_message)) {}
};
#endif

namespace torque {
namespace gpu {

namespace detail {
inline void check(tq_status st) {
  if (st == TQ_OK) return;
  const std::string msg = tq_last_error_string();
  if (st == TQ_ERR_INVALID || st == TQ_ERR_RANGE || st == TQ_ERR_UNSUPPORTED) throw Error(msg);
  throw std::runtime_error("torque_gb300: " + msg);
}

inline std::vector<int64_t> flat(const arma::uvec &v) {
  std::vector<int64_t> out(v.n_elem);
  for (arma::uword i = 0; i < v.n_elem; i++) out[i] = (int64_t)v(i);
  return out;
}

// rank x n matrix (column = block) -> the same memory as int64
inline std::vector<int64_t> flat(const arma::umat &m) {
  std::vector<int64_t> out(m.n_elem);
  for (arma::uword c = 0; c < m.n_cols; c++)
    for (arma::uword r = 0; r < m.n_rows; r++) out[c * m.n_rows + r] = (int64_t)m(r, c);
  return out;
}

template <typename T>
constexpr tq_dtype dtype() {
  static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value ||
                    std::is_same<T, __half>::value,
                "torque_gb300 supports float, double and half tensors");
  return std::is_same<T, float>::value ? TQ_F32 : std::is_same<T, double>::value ? TQ_F64 : TQ_F16;
}

inline tq_memkind kind_of(cudaMemcpyKind k) {
  return (k == cudaMemcpyHostToDevice || k == cudaMemcpyHostToHost) ? TQ_MEM_HOST : TQ_MEM_DEVICE;
}
}  // namespace detail

template <typename T>
class BlockSparseTensor {
 public:
  arma::uword rank = 0;
  arma::uvec dimension;
  arma::umat blocks_dimension;
  arma::umat index_tables;
  arma::umat begin_points;
  arma::umat end_points;
  arma::uvec block_n_elem;
  arma::uvec block_offsets;

  explicit BlockSparseTensor(const arma::uvec &dim) {
    const auto d = detail::flat(dim);
    detail::check(tq_bs_create_empty(detail::dtype<T>(), (int32_t)dim.n_elem, d.data(), &h_));
    refresh();
  }

  BlockSparseTensor(const T *source_data, const arma::umat &begin, const arma::umat &end,
                    const arma::uvec &total_dimension,
                    const cudaMemcpyKind kind = cudaMemcpyHostToDevice) {
    create(source_data, begin, end, total_dimension, nullptr, kind);
  }

  BlockSparseTensor(const T *source_data, const arma::umat &begin, const arma::umat &end,
                    const arma::uvec &total_dimension, const arma::umat &tables,
                    const cudaMemcpyKind kind = cudaMemcpyDeviceToDevice) {
    create(source_data, begin, end, total_dimension, &tables, kind);
  }

  // The raw move-in constructor (block_sparse.cuh:283-304): takes ownership of
  // `data`, a device buffer the caller allocated with cudaMalloc, without a
  // copy; the tensor frees it with cudaFree.  The redundant metadata
  // (blocks_dimension, block_n_elem, block_offsets) must agree with the boxes
  // (Error otherwise, and the buffer stays the caller's).
  BlockSparseTensor(T *data, arma::uword rank, arma::uvec &&dimension,
                    arma::umat &&blocks_dimension, arma::umat &&begin_points,
                    arma::umat &&end_points, arma::uvec &&block_n_elem,
                    arma::uvec &&block_offsets, arma::umat &&index_tables) {
    if (dimension.n_elem != rank) throw Error("Rank does not match");
    const int64_t nb = rank ? (int64_t)begin_points.n_cols : 0;
    for (int64_t k = 0; k < nb; k++) {
      arma::uword cnt = 1;
      for (arma::uword l = 0; l < rank; l++) {
        const arma::uword d = end_points(l, k) - begin_points(l, k) + 1;
        if (blocks_dimension(l, k) != d)
          throw Error("blocks_dimension does not match the begin and end points");
        cnt *= d;
      }
      if (block_n_elem(k) != cnt) throw Error("block_n_elem does not match the block boxes");
    }
    const auto d = detail::flat(dimension), b = detail::flat(begin_points),
               e = detail::flat(end_points), t = detail::flat(index_tables),
               off = detail::flat(block_offsets);
    detail::check(tq_bs_adopt(detail::dtype<T>(), (int32_t)rank, d.data(), nb, b.data(), e.data(),
                              index_tables.n_elem ? t.data() : nullptr,
                              block_offsets.n_elem ? off.data() : nullptr, data, &h_));
    refresh();
  }

  BlockSparseTensor(const BlockSparseTensor &o) {
    detail::check(tq_bs_clone(o.h_, nullptr, &h_));
    refresh();
  }
  BlockSparseTensor(BlockSparseTensor &&o) noexcept { swap(*this, o); }
  BlockSparseTensor &operator=(BlockSparseTensor &&o) noexcept {
    swap(*this, o);
    return *this;
  }
  BlockSparseTensor &operator=(const BlockSparseTensor &o) {
    BlockSparseTensor tmp(o);
    swap(*this, tmp);
    return *this;
  }
  ~BlockSparseTensor() {
    if (h_) tq_bs_destroy(h_);
  }

  friend void swap(BlockSparseTensor &a, BlockSparseTensor &b) noexcept {
    std::swap(a.h_, b.h_);
    std::swap(a.rank, b.rank);
    std::swap(a.dimension, b.dimension);
    std::swap(a.blocks_dimension, b.blocks_dimension);
    std::swap(a.index_tables, b.index_tables);
    std::swap(a.begin_points, b.begin_points);
    std::swap(a.end_points, b.end_points);
    std::swap(a.block_n_elem, b.block_n_elem);
    std::swap(a.block_offsets, b.block_offsets);
  }

  T to_number() const {
    T v;
    detail::check(tq_bs_to_number(h_, &v));
    return v;
  }

  void append_block(const T *source_data, const arma::uvec &begin_point,
                    const arma::uvec &end_point, const arma::uvec &index_table,
                    const cudaMemcpyKind kind = cudaMemcpyHostToDevice) {
    const auto b = detail::flat(begin_point), e = detail::flat(end_point),
               t = detail::flat(index_table);
    if (b.size() != rank || e.size() != rank) throw Error("Rank does not match");
    detail::check(tq_bs_append_blocks(h_, 1, b.data(), e.data(),
                                      t.size() == rank ? t.data() : nullptr, source_data,
                                      detail::kind_of(kind), nullptr));
    refresh();
  }

  void append_blocks(const T *const source_data, const arma::umat &begin,
                     const arma::umat &end, const arma::umat &tables,
                     const cudaMemcpyKind kind = cudaMemcpyHostToDevice) {
    const auto b = detail::flat(begin), e = detail::flat(end), t = detail::flat(tables);
    detail::check(tq_bs_append_blocks(h_, (int64_t)begin.n_cols, b.data(), e.data(),
                                      t.size() == b.size() ? t.data() : nullptr, source_data,
                                      detail::kind_of(kind), nullptr));
    refresh();
  }

  void modify(const arma::uvec &indices, const T number) {
    if (indices.n_elem != rank) throw Error("Rank does not match");
    const auto i = detail::flat(indices);
    detail::check(tq_bs_modify(h_, i.data(), &number));
    refresh();
  }

  T query(const arma::uvec &indices) const {
    if (indices.n_elem != rank) throw Error("Rank does not match");
    const auto i = detail::flat(indices);
    T v;
    detail::check(tq_bs_query(h_, i.data(), &v));
    return v;
  }

  // contract(handle, tensor, contracting_indices): the handle is accepted for
  // source compatibility and not used.
  template <typename Handle>
  BlockSparseTensor contract(Handle, const BlockSparseTensor &tensor,
                             const arma::umat &contracting_indices,
                             const tq_contract_opts *opts = nullptr) const {
    return contract(tensor, contracting_indices, opts);
  }

  BlockSparseTensor contract(const BlockSparseTensor &tensor,
                             const arma::umat &contracting_indices,
                             const tq_contract_opts *opts = nullptr) const {
    if (contracting_indices.n_elem && contracting_indices.n_cols != 2)
      throw Error("contracting indices must be an n x 2 matrix");
    const arma::uword n = contracting_indices.n_elem ? contracting_indices.n_rows : 0;
    std::vector<int64_t> al(n), bl(n);
    for (arma::uword k = 0; k < n; k++) {
      al[k] = (int64_t)contracting_indices(k, 0);
      bl[k] = (int64_t)contracting_indices(k, 1);
    }
    tq_bs *out = nullptr;
    detail::check(tq_bs_contract(h_, tensor.h_, (int32_t)n, al.data(), bl.data(), opts, nullptr,
                                 &out));
    return BlockSparseTensor(out);
  }

  BlockSparseTensor hard_transpose(const arma::uvec &permutation) const {
    if (permutation.n_elem != rank)
      throw Error("The number of permutation does not match the rank of tensor");
    const auto p = detail::flat(permutation);
    tq_bs *out = nullptr;
    detail::check(tq_bs_hard_transpose(h_, p.data(), nullptr, &out));
    return BlockSparseTensor(out);
  }

  BlockSparseTensor slice(const arma::uvec &divisor) const {
    const auto d = detail::flat(divisor);
    tq_bs *out = nullptr;
    detail::check(tq_bs_slice(h_, d.data(), nullptr, &out));
    return BlockSparseTensor(out);
  }

  // Legs `leg` and `leg`+1 fused into one (an extension: the reference has no
  // leg fusion).  bounds_a / bounds_b: sector boundaries of the two legs (first
  // 0, last the leg's dimension); pair_offset(a, b): where sector pair (a, b)
  // starts in the fused leg.  See tq_bs_fuse_legs.
  BlockSparseTensor fuse_legs(arma::uword leg, const arma::uvec &bounds_a,
                              const arma::uvec &bounds_b, const arma::umat &pair_offset) const {
    if (leg + 1 >= rank) throw Error("legs to fuse out of range");
    if (pair_offset.n_rows + 1 != bounds_a.n_elem || pair_offset.n_cols + 1 != bounds_b.n_elem)
      throw Error("pair_offset must be (sectors of a) x (sectors of b)");
    const auto ba = detail::flat(bounds_a), bb = detail::flat(bounds_b),
               off = detail::flat(pair_offset);
    tq_bs *out = nullptr;
    detail::check(tq_bs_fuse_legs(h_, (int32_t)leg, (int64_t)ba.size() - 1, ba.data(),
                                  (int64_t)bb.size() - 1, bb.data(), off.data(), nullptr, &out));
    return BlockSparseTensor(out);
  }

  // Inverse of fuse_legs (an extension): leg `leg` split back into two legs,
  // with the bounds and pair offsets that fused them.  See tq_bs_split_leg.
  BlockSparseTensor split_leg(arma::uword leg, const arma::uvec &bounds_a,
                              const arma::uvec &bounds_b, const arma::umat &pair_offset) const {
    if (leg >= rank) throw Error("leg to split out of range");
    if (pair_offset.n_rows + 1 != bounds_a.n_elem || pair_offset.n_cols + 1 != bounds_b.n_elem)
      throw Error("pair_offset must be (sectors of a) x (sectors of b)");
    const auto ba = detail::flat(bounds_a), bb = detail::flat(bounds_b),
               off = detail::flat(pair_offset);
    tq_bs *out = nullptr;
    detail::check(tq_bs_split_leg(h_, (int32_t)leg, (int64_t)ba.size() - 1, ba.data(),
                                  (int64_t)bb.size() - 1, bb.data(), off.data(), nullptr, &out));
    return BlockSparseTensor(out);
  }

  // A charge-conserving tensor (an extension): leg l has the sectors
  // charges[l] / sizes[l] laid out in order and direction directions(l) (+1 in,
  // -1 out); blocks for every sector tuple with sum(direction * charge) ==
  // total (mod modulus for Z_n, 0 = U(1)), leg 0 fastest; data in block order,
  // or zeros when src is NULL.  See tq_bs_create_charges.
  static BlockSparseTensor from_charges(const std::vector<arma::Col<long long>> &charges,
                                        const std::vector<arma::uvec> &sizes,
                                        const std::vector<int> &directions, const T *src,
                                        long long total = 0, long long modulus = 0,
                                        cudaMemcpyKind kind = cudaMemcpyHostToDevice) {
    if (charges.size() != sizes.size() || charges.size() != directions.size())
      throw Error("one charge list, size list and direction per leg");
    std::vector<int64_t> ns, q, sz;
    std::vector<int32_t> dir;
    for (size_t l = 0; l < charges.size(); l++) {
      if (charges[l].n_elem != sizes[l].n_elem) throw Error("charges and sizes must pair up");
      ns.push_back((int64_t)charges[l].n_elem);
      for (arma::uword s = 0; s < charges[l].n_elem; s++) {
        q.push_back((int64_t)charges[l](s));
        sz.push_back((int64_t)sizes[l](s));
      }
      dir.push_back(directions[l]);
    }
    tq_bs *out = nullptr;
    detail::check(tq_bs_create_charges(detail::dtype<T>(), (int32_t)charges.size(), ns.data(),
                                       q.data(), sz.data(), dir.data(), total, modulus, src,
                                       detail::kind_of(kind), nullptr, &out));
    return BlockSparseTensor(out);
  }

  // New values for every element (an extension, tq_bs_set_data): n_elem
  // elements in the tensor's layout, from host or device memory.
  void set_data(const T *src, cudaMemcpyKind kind = cudaMemcpyHostToDevice) {
    detail::check(tq_bs_set_data(h_, src, detail::kind_of(kind), nullptr));
  }

  // Block-level truncated SVD (an extension, float64 tensors; tq_bs_svd):
  // row_legs against the other legs; U[row legs..., bond], S[bond] and
  // V[bond, column legs...], keeping at most max_keep values (0: all) above
  // cutoff times the largest.
  std::tuple<BlockSparseTensor, BlockSparseTensor, BlockSparseTensor> svd(
      const arma::uvec &row_legs, long long max_keep = 0, double cutoff = 0.0) const {
    const auto rl = detail::flat(row_legs);
    tq_bs *u = nullptr, *s = nullptr, *v = nullptr;
    detail::check(tq_bs_svd(h_, (int32_t)rl.size(), rl.data(), (int64_t)max_keep, cutoff, nullptr,
                            &u, &s, &v));
    return std::make_tuple(BlockSparseTensor(u), BlockSparseTensor(s), BlockSparseTensor(v));
  }

  // Block-level QR (an extension, float64 tensors; tq_bs_qr): Q[row legs...,
  // bond] with orthonormal columns and R[bond, column legs...], upper
  // trapezoidal in each charge class.
  std::pair<BlockSparseTensor, BlockSparseTensor> qr(const arma::uvec &row_legs) const {
    const auto rl = detail::flat(row_legs);
    tq_bs *q = nullptr, *r = nullptr;
    detail::check(tq_bs_qr(h_, (int32_t)rl.size(), rl.data(), nullptr, &q, &r));
    return std::make_pair(BlockSparseTensor(q), BlockSparseTensor(r));
  }

  // the underlying handle, for calls of the C ABI not wrapped here
  tq_bs *handle() const { return h_; }

 private:
  explicit BlockSparseTensor(tq_bs *h) : h_(h) { refresh(); }

  void create(const T *src, const arma::umat &begin, const arma::umat &end,
              const arma::uvec &dim, const arma::umat *tables, cudaMemcpyKind kind) {
    const auto d = detail::flat(dim), b = detail::flat(begin), e = detail::flat(end);
    std::vector<int64_t> t;
    if (tables) t = detail::flat(*tables);
    const int64_t nb = dim.n_elem ? (int64_t)begin.n_cols : 0;
    detail::check(tq_bs_create(detail::dtype<T>(), (int32_t)dim.n_elem, d.data(), nb, b.data(),
                               e.data(), tables ? t.data() : nullptr, src,
                               detail::kind_of(kind), nullptr, &h_));
    refresh();
  }

  void refresh() {
    tq_dtype dt;
    int32_t r = 0;
    int64_t nb = 0, ne = 0;
    detail::check(tq_bs_shape(h_, &dt, &r, &nb, &ne));
    std::vector<int64_t> d(r), b(nb * r), e(nb * r), t(nb * r), off(nb);
    detail::check(tq_bs_metadata(h_, d.data(), b.data(), e.data(), t.data(), off.data()));
    rank = (arma::uword)r;
    dimension = arma::uvec(rank);
    for (int32_t l = 0; l < r; l++) dimension(l) = (arma::uword)d[l];
    begin_points = arma::umat(rank, nb);
    end_points = arma::umat(rank, nb);
    index_tables = arma::umat(rank, nb);
    blocks_dimension = arma::umat(rank, nb);
    block_n_elem = arma::uvec(nb);
    block_offsets = arma::uvec(nb);
    for (int64_t k = 0; k < nb; k++) {
      arma::uword cnt = 1;
      for (int32_t l = 0; l < r; l++) {
        begin_points(l, k) = (arma::uword)b[k * r + l];
        end_points(l, k) = (arma::uword)e[k * r + l];
        index_tables(l, k) = (arma::uword)t[k * r + l];
        blocks_dimension(l, k) = end_points(l, k) - begin_points(l, k) + 1;
        cnt *= blocks_dimension(l, k);
      }
      block_n_elem(k) = cnt;
      block_offsets(k) = (arma::uword)off[k];
    }
  }

  tq_bs *h_ = nullptr;
};

}  // namespace gpu
}  // namespace torque
