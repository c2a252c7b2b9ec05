// Block lists of tensors with a charge-conserving symmetry (U(1) or Z_n).
//
// Torque has no charges: its callers map symmetry sectors to coordinate boxes
// themselves (src/tensor/block_sparse.h:109-145).  These entry points do that
// mapping for C and C++ callers: each leg is cut into contiguous coordinate
// ranges, one per sector, in the order the sectors are given; a block exists
// for every tuple of sectors whose signed charges add up to the total; blocks
// are listed in column-major order of the sector indices (leg 0 fastest, the
// reference's index convention, src/util/space.h:11-24).
#include <cstring>
#include <vector>

#include "tq_internal.h"

namespace tq {

// Sector tuples, leg 0 fastest, with sum(direction * charge) == total (mod
// modulus when modulus > 0).  U(1) enumeration prunes a partial tuple when the
// legs left cannot bring its charge back to the total.
static tq_status charge_tuples(int32_t rank, const int64_t *n_sectors, const int64_t *charges,
                               const int32_t *directions, int64_t total, int64_t modulus,
                               std::vector<int32_t> &out) {
  std::vector<const int64_t *> q(rank);
  int64_t off = 0;
  for (int32_t l = 0; l < rank; l++) {
    if (n_sectors[l] <= 0) return fail(TQ_ERR_INVALID, "a leg without sectors");
    if (directions[l] != 1 && directions[l] != -1)
      return fail(TQ_ERR_INVALID, "leg directions must be +1 or -1");
    q[l] = charges + off;
    off += n_sectors[l];
  }
  // lo[l] / hi[l]: the charge range legs 0..l-1 can still add (U(1) pruning)
  std::vector<int64_t> lo(rank + 1, 0), hi(rank + 1, 0);
  for (int32_t l = 0; l < rank; l++) {
    int64_t mn = INT64_MAX, mx = INT64_MIN;
    for (int64_t s = 0; s < n_sectors[l]; s++) {
      const int64_t v = directions[l] * q[l][s];
      mn = v < mn ? v : mn;
      mx = v > mx ? v : mx;
    }
    lo[l + 1] = lo[l] + mn;
    hi[l + 1] = hi[l] + mx;
  }
  std::vector<int32_t> idx(rank, 0);
  // depth-first from the last leg (outermost) to leg 0 (innermost)
  struct Rec {
    static void go(int32_t l, int64_t c, int32_t rank, const std::vector<const int64_t *> &q,
                   const int64_t *ns, const int32_t *dir, int64_t total, int64_t mod,
                   const std::vector<int64_t> &lo, const std::vector<int64_t> &hi,
                   std::vector<int32_t> &idx, std::vector<int32_t> &out) {
      if (l < 0) {
        const bool ok = mod > 0 ? ((c - total) % mod + mod) % mod == 0 : c == total;
        if (ok) out.insert(out.end(), idx.begin(), idx.end());
        return;
      }
      for (int64_t s = 0; s < ns[l]; s++) {
        const int64_t cc = c + dir[l] * q[l][s];
        if (mod == 0 && (total - cc < lo[l] || total - cc > hi[l])) continue;
        idx[l] = (int32_t)s;
        go(l - 1, cc, rank, q, ns, dir, total, mod, lo, hi, idx, out);
      }
    }
  };
  // the recursion's outer loop is the last leg, so leg 0 varies fastest
  Rec::go(rank - 1, 0, rank, q, n_sectors, directions, total, modulus, lo, hi, idx, out);
  return TQ_OK;
}

static tq_status charge_boxes(int32_t rank, const int64_t *n_sectors, const int64_t *charges,
                              const int64_t *sizes, const int32_t *directions, int64_t total,
                              int64_t modulus, std::vector<int64_t> &dim,
                              std::vector<int64_t> &begin, std::vector<int64_t> &end) {
  if (rank <= 0 || rank > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "rank outside 1..12");
  if (!n_sectors || !charges || !sizes || !directions) return fail(TQ_ERR_INVALID, "NULL argument");
  if (modulus < 0) return fail(TQ_ERR_INVALID, "negative modulus");
  std::vector<int32_t> tup;
  TQ_CHECK(charge_tuples(rank, n_sectors, charges, directions, total, modulus, tup));
  std::vector<std::vector<int64_t>> start(rank);
  dim.assign(rank, 0);
  int64_t off = 0;
  for (int32_t l = 0; l < rank; l++) {
    for (int64_t s = 0; s < n_sectors[l]; s++) {
      if (sizes[off + s] <= 0) return fail(TQ_ERR_INVALID, "sector sizes must be positive");
      start[l].push_back(dim[l]);
      dim[l] += sizes[off + s];
    }
    off += n_sectors[l];
  }
  const size_t nb = tup.size() / (size_t)rank;
  begin.resize(tup.size());
  end.resize(tup.size());
  for (size_t b = 0; b < nb; b++) {
    int64_t o = 0;
    for (int32_t l = 0; l < rank; l++) {
      const int32_t s = tup[b * rank + l];
      begin[b * rank + l] = start[l][s];
      end[b * rank + l] = start[l][s] + sizes[o + s] - 1;
      o += n_sectors[l];
    }
  }
  return TQ_OK;
}

}  // namespace tq

using namespace tq;

extern "C" {

tq_status tq_charge_blocks(int32_t rank, const int64_t *n_sectors, const int64_t *charges,
                           const int64_t *sizes, const int32_t *directions, int64_t total,
                           int64_t modulus, int64_t cap, int64_t *n_blocks,
                           int64_t *begin_points, int64_t *end_points) {
  if (!n_blocks) return fail(TQ_ERR_INVALID, "NULL argument");
  std::vector<int64_t> dim, b, e;
  TQ_CHECK(charge_boxes(rank, n_sectors, charges, sizes, directions, total, modulus, dim, b, e));
  const int64_t nb = (int64_t)(b.size() / (size_t)rank);
  *n_blocks = nb;
  if (cap >= nb && nb > 0) {
    if (!begin_points || !end_points) return fail(TQ_ERR_INVALID, "NULL output arrays");
    std::memcpy(begin_points, b.data(), b.size() * 8);
    std::memcpy(end_points, e.data(), e.size() * 8);
  }
  return TQ_OK;
}

tq_status tq_bs_create_charges(tq_dtype dtype, int32_t rank, const int64_t *n_sectors,
                               const int64_t *charges, const int64_t *sizes,
                               const int32_t *directions, int64_t total, int64_t modulus,
                               const void *data, tq_memkind kind, tq_stream stream,
                               tq_bs **out) {
  if (!out) return fail(TQ_ERR_INVALID, "out is NULL");
  std::vector<int64_t> dim, b, e;
  TQ_CHECK(charge_boxes(rank, n_sectors, charges, sizes, directions, total, modulus, dim, b, e));
  const int64_t nb = (int64_t)(b.size() / (size_t)rank);
  if (!data)
    return tq_bs_create_zeros(dtype, rank, dim.data(), nb, b.data(), e.data(), nullptr, stream,
                              out);
  return tq_bs_create(dtype, rank, dim.data(), nb, b.data(), e.data(), nullptr, data, kind, stream,
                      out);
}

}  // extern "C"
