// Internal types shared by the CUDA translation units of libtorque_gb300.
//
// Data model (follows torque::gpu::BlockSparseTensor, src/gpu/block_sparse.cuh:143-178):
// a tensor is a list of boxes with inclusive begin/end points per leg; the
// metadata matrices are rank x n_blocks with one column per block, i.e. block b,
// leg l lives at [b*rank + l].  Block data is stored back to back in one device
// buffer; block_offsets is the exclusive scan of the block element counts.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "torque_gb300.h"

#define TQ_MAXR 12  // maximum rank handled on device (the reference uses 10)

namespace tq {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
tq_status fail(tq_status st, const std::string &msg);
tq_status cuda_fail(cudaError_t e, const char *what);

#define TQ_CUDA(call)                                          \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return ::tq::cuda_fail(e_, #call);  \
  } while (0)

#define TQ_CHECK(call)                   \
  do {                                   \
    tq_status s_ = (call);               \
    if (s_ != TQ_OK) return s_;          \
  } while (0)

// ---------------------------------------------------------------- tracing
// A named NVTX range over a host scope: the phases of a contraction (plan,
// operand preparation, GEMM), transposes and batch runs show up on a profiler's
// timeline, and `ncu --nvtx --nvtx-include "tq_gemm/"` selects the kernels
// launched inside one.  Ranges are flat (never nested).  Without a tool
// attached the calls do nothing.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// ---------------------------------------------------------------- memory
// Stream-ordered device allocation; every call goes through here so that an
// allocation hook (used by fault-injection tests) can refuse it.
tq_status dev_alloc(void **p, size_t bytes, cudaStream_t s);
void dev_free(void *p, cudaStream_t s);

template <typename T>
struct DevArray {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DevArray() = default;
  DevArray(const DevArray &) = delete;
  DevArray &operator=(const DevArray &) = delete;
  DevArray(DevArray &&o) noexcept { *this = std::move(o); }
  DevArray &operator=(DevArray &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p; n = o.n; s = o.s;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DevArray() { release(); }
  tq_status alloc(size_t count, cudaStream_t stream) {
    release();
    s = stream;
    n = count;
    if (count == 0) return TQ_OK;
    return dev_alloc((void **)&p, count * sizeof(T), stream);
  }
  void release() {
    if (p) dev_free(p, s);
    p = nullptr;
    n = 0;
  }
};

size_t dtype_size(tq_dtype t);

// Every kernel launch of the library goes through this counter (reported by
// tq_debug_kernel_launches).
void count_launch();

// ---------------------------------------------------------------- kernels' views
struct DevBS {
  int32_t rank;
  int64_t nb;
  const int64_t *begin;
  const int64_t *end;
  const int64_t *strides;
  const int64_t *offsets;
  const void *data;
};

// Contracted legs in pair order and the free legs in ascending order.
struct LegSpec {
  int32_t nc, nfa, nfb, rank_a, rank_b;
  int32_t al[TQ_MAXR], bl[TQ_MAXR];
  int32_t fa[TQ_MAXR], fb[TQ_MAXR];
};

}  // namespace tq

// ---------------------------------------------------------------- tensor object
struct tq_bs {
  tq_dtype dtype = TQ_F64;
  int32_t rank = 0;
  int device = 0;
  std::vector<int64_t> dimension;
  int64_t nb = 0;
  // host metadata (authoritative when host_valid)
  std::vector<int64_t> h_begin, h_end, h_strides, h_offsets;
  bool host_valid = true;
  // device metadata: begin | end | strides (nb*rank each) | offsets (nb)
  tq::DevArray<int64_t> d_meta;
  bool dev_valid = false;
  // data
  void *data = nullptr;
  int64_t n_elem = 0;      // elements in use
  int64_t capacity = 0;    // elements allocated
  cudaStream_t alloc_stream = nullptr;
  bool adopted = false;    // data is a caller's cudaMalloc buffer (tq_bs_adopt): cudaFree

  tq::DevBS view() const {
    tq::DevBS v;
    v.rank = rank;
    v.nb = nb;
    v.begin = d_meta.p;
    v.end = d_meta.p ? d_meta.p + nb * rank : nullptr;
    v.strides = d_meta.p ? d_meta.p + 2 * nb * rank : nullptr;
    v.offsets = d_meta.p ? d_meta.p + 3 * nb * rank : nullptr;
    v.data = data;
    return v;
  }
};

namespace tq {
tq_status sync_device_meta(tq_bs *t, cudaStream_t s);
tq_status sync_host_meta(tq_bs *t, cudaStream_t s);
tq_status alloc_data(tq_bs *t, int64_t n_elem, cudaStream_t s);
tq_bs *new_tensor(tq_dtype dt, int32_t rank, const int64_t *dimension);
}  // namespace tq
