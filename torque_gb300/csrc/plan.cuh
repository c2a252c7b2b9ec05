// The plan of one contraction: everything the numeric stage needs, resident on
// the device, produced by the symbolic stage.
#pragma once
#include <memory>

#include "gemm.cuh"
#include "ozaki.cuh"
#include "tq_internal.h"

namespace tq {
// Device arrays behind a NativeWork (split-K work list of the native kernel).
struct NativeWorkDev {
  DevArray<int32_t> chunks;
  DevArray<int64_t> kfused, work_start, split_start, split_off;
  DevArray<uint8_t> scratch;
  NativeWork w;
};
}  // namespace tq

struct tq_plan {
  const tq_bs *A = nullptr, *B = nullptr;
  tq_bs *C = nullptr;  // owned by the caller
  void *out = nullptr; // where the numeric stage writes (null: C's own buffer)
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
  tq::NativeWorkDev nat;                  // native kernel work list (all outputs)
  // tensor-core (sliced) forms
  int32_t slices = 0;
  bool tc = false;
  tq::DevArray<int64_t> keyA, keyB;            // free-box class key per block
  tq::DevArray<int64_t> rowA, rowB;            // per key: exponent table offset
  tq::DevArray<int64_t> rowstartA, rowstartB;  // per block: first row
  tq::DevArray<int64_t> tilestartA, tilestartB;
  tq::DevArray<int64_t> unitA, unitB;          // per block: slice offset / 256 B
  tq::DevArray<int64_t> ksum, tc_tile_start;
  tq::DevArray<int32_t> expA, expB, nk_pair;
  tq::DevArray<uint8_t> sliceA, sliceB;
  int64_t rowsA = 0, rowsB = 0, tilesA = 0, tilesB = 0, nexpA = 0, nexpB = 0, tc_tiles = 0;
  int32_t tile_n = 0;
  int64_t KA = 0, KB = 0;  // free-box key ranges (tensor-core plans, reduced layout)
  bool keys = false;       // keyA/keyB were made
  bool sched_ok = true;    // false after a failed reschedule: execute refuses
  // bumped by every reschedule: a batch built from this plan holds device
  // copies of the schedule's array pointers and refuses to run once it changed
  uint64_t sched_gen = 0;
  // block grouping: native 64x64 tiles of the outputs sent to plain FP64
  tq::DevArray<int64_t> hyb_tile_start;
  int64_t hyb_tiles = 0;
  tq::NativeWorkDev hyb;
  tq::DevArray<tq::OzPairRec> pair_tab;  // pairs in GEMM order (tensor-core forms)
  // class layout of the tensor-core forms (see OzClassOut)
  bool classes = false;
  int64_t n_cls = 0;
  tq::DevArray<tq::OzClassOut> cls_out;
  tq::DevArray<tq::OzRowMap> rmapA, rmapB;
  tq::DevArray<tq::OzClassItem> itemsA, itemsB;
  tq::DevArray<int32_t> blkA, blkB;
  tq::DevArray<int64_t> cls_offs;
  tq::OzJob tc_job{};              // this contraction as one job
  tq::OzSide tc_side[2]{};         // its A and B operand sides
  tq::OzBatchDev tcb;              // the same as a batch of one, on the device
  // optional phase timing (events on the launching stream)
  bool profile = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  ~tq_plan() {
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  }
};

namespace tq {
tq_status run_hybrid_native(tq_plan *P, cudaStream_t s);
tq_status plan_run(tq_plan *P, cudaStream_t s);
tq_status plan_check(tq_plan *P, cudaStream_t s);
tq_status plan_reschedule(tq_plan *P, const tq_contract_opts &o, cudaStream_t s);
tq_status validate_legs(const tq_bs *A, const tq_bs *B, int32_t n_legs, const int64_t *a_legs,
                        const int64_t *b_legs, LegSpec &L);
}
