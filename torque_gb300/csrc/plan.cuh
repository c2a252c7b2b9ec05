// The plan of one contraction: everything the numeric stage needs, resident on
// the device, produced by the symbolic stage.
#pragma once
#include <memory>

#include "tq_internal.h"

struct tq_plan {
  const tq_bs *A = nullptr, *B = nullptr;
  tq_bs *C = nullptr;  // owned by the caller
  tq::LegSpec L;
  tq_contract_opts opts;
  int64_t n_pairs = 0, n_out = 0, n_tiles = 0, n_chunks = 0;
  double flops = 0.0;
  tq::DevArray<int32_t> pa, pb;           // pairs, reference order
  tq::DevArray<int64_t> seg;              // [n_out+1]
  tq::DevArray<int64_t> perm;             // reduced layout: pairs sorted by output box
  tq::DevArray<int64_t> tile_start;       // [n_out+1]
  tq::DevArray<int64_t> chunk_start;      // rank-0 results
  tq::DevArray<double> partials;          // rank-0 results (float partials use the low half)
};

namespace tq {
tq_status validate_legs(const tq_bs *A, const tq_bs *B, int32_t n_legs, const int64_t *a_legs,
                        const int64_t *b_legs, LegSpec &L);
}
