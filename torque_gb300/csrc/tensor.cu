// Tensor lifecycle, element access and metadata of the block-sparse tensor.
// Mirrors torque::gpu::BlockSparseTensor (src/gpu/block_sparse.cuh:143-552,
// 1124-1176); errors become status codes instead of exit().
#include <cuda_fp16.h>
#include <cstring>
#include <atomic>
#include <mutex>

#include "tq_internal.h"

namespace tq {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_alloc_budget{-1};
static std::atomic<int64_t> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const std::string &msg) { g_last_error = msg; }

tq_status fail(tq_status st, const std::string &msg) {
  g_last_error = msg;
  return st;
}

tq_status cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string("CUDA error ") + cudaGetErrorName(e) + " (" +
                 cudaGetErrorString(e) + ") in " + what;
  if (e == cudaErrorMemoryAllocation) return TQ_ERR_OOM;
  return TQ_ERR_CUDA;
}

// The library's own stream-ordered memory pool per device.  Freed memory stays
// in the pool (release threshold: unlimited), so a contraction that allocates
// tens of GB again and again does not map and unmap pages every time; the
// process's default pool is left as it was.  tq_release_cached_memory trims it.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pools[128] = {nullptr};

static tq_status device_pool(cudaMemPool_t *pool) {
  int dev = 0;
  TQ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(TQ_ERR_UNSUPPORTED, "device ordinal above 127");
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pools[dev]) {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pl = nullptr;
    TQ_CUDA(cudaMemPoolCreate(&pl, &props));
    uint64_t keep = UINT64_MAX;
    TQ_CUDA(cudaMemPoolSetAttribute(pl, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pools[dev] = pl;
  }
  *pool = g_pools[dev];
  return TQ_OK;
}

tq_status dev_alloc(void **p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  int64_t b = g_alloc_budget.load();
  if (b >= 0) {
    if (b == 0) return fail(TQ_ERR_OOM, "device allocation refused by the test hook");
    g_alloc_budget.store(b - 1);
  }
  if (bytes == 0) bytes = 16;
  cudaMemPool_t pool = nullptr;
  TQ_CHECK(device_pool(&pool));
  cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, s);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_fail(e, "cudaMallocFromPoolAsync");
  }
  return TQ_OK;
}

void dev_free(void *p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

size_t dtype_size(tq_dtype t) { return t == TQ_F16 ? 2 : t == TQ_F32 ? 4 : 8; }

tq_bs *new_tensor(tq_dtype dt, int32_t rank, const int64_t *dimension) {
  tq_bs *t = new tq_bs();
  t->dtype = dt;
  t->rank = rank;
  t->dimension.assign(dimension, dimension + rank);
  cudaGetDevice(&t->device);
  return t;
}

// Frees a tensor's value buffer: the library pool's stream-ordered free, or,
// for a buffer adopted from the caller (tq_bs_adopt), cudaFree after the work
// queued on the device (a copy out of it on any stream) has finished.
static void free_data(tq_bs *t) {
  if (t->data) {
    if (t->adopted) {
      cudaDeviceSynchronize();
      cudaFree(t->data);
    } else {
      dev_free(t->data, t->alloc_stream);
    }
  }
  t->data = nullptr;
  t->adopted = false;
}

tq_status alloc_data(tq_bs *t, int64_t n_elem, cudaStream_t s) {
  free_data(t);
  t->alloc_stream = s;
  int64_t cap = n_elem > 0 ? n_elem : 1;
  TQ_CHECK(dev_alloc(&t->data, (size_t)cap * dtype_size(t->dtype), s));
  t->capacity = cap;
  t->n_elem = n_elem;
  return TQ_OK;
}

tq_status sync_device_meta(tq_bs *t, cudaStream_t s) {
  if (t->dev_valid) return TQ_OK;
  const size_t nr = (size_t)t->nb * t->rank;
  const size_t n = 3 * nr + (size_t)t->nb;
  TQ_CHECK(t->d_meta.alloc(n, s));
  if (n) {
    std::vector<int64_t> h(n);
    if (nr) {
      std::memcpy(h.data(), t->h_begin.data(), nr * 8);
      std::memcpy(h.data() + nr, t->h_end.data(), nr * 8);
      std::memcpy(h.data() + 2 * nr, t->h_strides.data(), nr * 8);
    }
    if (t->nb) std::memcpy(h.data() + 3 * nr, t->h_offsets.data(), t->nb * 8);
    TQ_CUDA(cudaMemcpyAsync(t->d_meta.p, h.data(), n * 8, cudaMemcpyHostToDevice, s));
    // the host vector dies here: make the copy complete before returning
    TQ_CUDA(cudaStreamSynchronize(s));
  }
  t->dev_valid = true;
  return TQ_OK;
}

tq_status sync_host_meta(tq_bs *t, cudaStream_t s) {
  if (t->host_valid) return TQ_OK;
  const size_t nr = (size_t)t->nb * t->rank;
  const size_t n = 3 * nr + (size_t)t->nb;
  std::vector<int64_t> h(n);
  if (n) {
    TQ_CUDA(cudaMemcpyAsync(h.data(), t->d_meta.p, n * 8, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaStreamSynchronize(s));
  }
  t->h_begin.assign(h.begin(), h.begin() + nr);
  t->h_end.assign(h.begin() + nr, h.begin() + 2 * nr);
  t->h_strides.assign(h.begin() + 2 * nr, h.begin() + 3 * nr);
  t->h_offsets.assign(h.begin() + 3 * nr, h.end());
  t->host_valid = true;
  return TQ_OK;
}

static tq_status check_boxes(int32_t rank, const int64_t *dimension, int64_t n,
                             const int64_t *b, const int64_t *e) {
  for (int64_t k = 0; k < n; k++)
    for (int32_t l = 0; l < rank; l++) {
      int64_t lo = b[k * rank + l], hi = e[k * rank + l];
      if (lo < 0 || hi < lo || hi >= dimension[l])
        return fail(TQ_ERR_INVALID, "block " + std::to_string(k) + " leg " +
                                        std::to_string(l) + ": box [" + std::to_string(lo) +
                                        ", " + std::to_string(hi) + "] outside dimension " +
                                        std::to_string(dimension[l]));
    }
  return TQ_OK;
}

static tq_status append_meta(tq_bs *t, int64_t n, const int64_t *b, const int64_t *e,
                             const int64_t *tables, int64_t *added_elems) {
  const int32_t r = t->rank;
  int64_t total = 0;
  for (int64_t k = 0; k < n; k++) {
    int64_t cnt = 1, stride = 1;
    for (int32_t l = 0; l < r; l++) {
      const int64_t d = e[k * r + l] - b[k * r + l] + 1;
      t->h_begin.push_back(b[k * r + l]);
      t->h_end.push_back(e[k * r + l]);
      t->h_strides.push_back(tables ? tables[k * r + l] : stride);
      stride *= d;
      cnt *= d;
    }
    t->h_offsets.push_back(t->n_elem + total);
    total += cnt;
  }
  t->nb += n;
  *added_elems = total;
  t->dev_valid = false;
  return TQ_OK;
}

}  // namespace tq

using namespace tq;

extern "C" tq_status tq_release_cached_memory(void) {
  std::lock_guard<std::mutex> lk(tq::g_pool_mu);
  for (int d = 0; d < 128; d++) {
    if (!tq::g_pools[d]) continue;
    int cur = 0;
    TQ_CUDA(cudaGetDevice(&cur));
    TQ_CUDA(cudaSetDevice(d));
    const cudaError_t e1 = cudaDeviceSynchronize();
    const cudaError_t e2 = cudaMemPoolTrimTo(tq::g_pools[d], 0);
    TQ_CUDA(cudaSetDevice(cur));
    TQ_CUDA(e1);
    TQ_CUDA(e2);
  }
  return TQ_OK;
}

extern "C" {

const char *tq_last_error_string(void) { return g_last_error.c_str(); }

void tq_debug_fail_alloc_after(int64_t after) { g_alloc_budget.store(after); }

int64_t tq_debug_kernel_launches(void) { return g_launches.load(); }

tq_status tq_bs_create_empty(tq_dtype dtype, int32_t rank, const int64_t *dimension,
                             tq_bs **out) {
  if (!out) return fail(TQ_ERR_INVALID, "out is NULL");
  if (rank < 0 || rank > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "rank outside 0..12");
  if (rank && !dimension) return fail(TQ_ERR_INVALID, "dimension is NULL");
  if (dtype != TQ_F32 && dtype != TQ_F64 && dtype != TQ_F16)
    return fail(TQ_ERR_INVALID, "unknown dtype");
  tq_bs *t = new_tensor(dtype, rank, dimension);
  // The reference allocates one zeroed element (block_sparse.cuh:180-187);
  // for rank 0 it is the scalar.
  tq_status st = alloc_data(t, rank == 0 ? 1 : 0, nullptr);
  if (st == TQ_OK) {
    cudaError_t e = cudaMemsetAsync(t->data, 0, dtype_size(dtype), nullptr);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemsetAsync");
  }
  if (st != TQ_OK) {
    tq_bs_destroy(t);
    return st;
  }
  *out = t;
  return TQ_OK;
}

tq_status tq_bs_create(tq_dtype dtype, int32_t rank, const int64_t *dimension, int64_t n_blocks,
                       const int64_t *begin_points, const int64_t *end_points,
                       const int64_t *index_tables, const void *data, tq_memkind kind,
                       tq_stream stream, tq_bs **out) {
  if (!out) return fail(TQ_ERR_INVALID, "out is NULL");
  if (n_blocks < 0) return fail(TQ_ERR_INVALID, "negative block count");
  if (!data) return fail(TQ_ERR_INVALID, "Source data not allocated!");
  if (rank == 0) {
    tq_bs *t = nullptr;
    TQ_CHECK(tq_bs_create_empty(dtype, 0, nullptr, &t));
    cudaError_t e = cudaMemcpyAsync(t->data, data, dtype_size(dtype),
                                    kind == TQ_MEM_HOST ? cudaMemcpyHostToDevice
                                                        : cudaMemcpyDeviceToDevice,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess && kind == TQ_MEM_HOST) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) {
      tq_bs_destroy(t);
      return cuda_fail(e, "cudaMemcpyAsync");
    }
    *out = t;
    return TQ_OK;
  }
  if (n_blocks && (!begin_points || !end_points))
    return fail(TQ_ERR_INVALID, "begin/end points are NULL");
  if (rank < 0 || rank > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "rank outside 0..12");
  TQ_CHECK(check_boxes(rank, dimension, n_blocks, begin_points, end_points));
  tq_bs *t = new_tensor(dtype, rank, dimension);
  int64_t added = 0;
  append_meta(t, n_blocks, begin_points, end_points, index_tables, &added);
  tq_status st = alloc_data(t, added, (cudaStream_t)stream);
  if (st == TQ_OK && added) {
    cudaError_t e = cudaMemcpyAsync(t->data, data, (size_t)added * dtype_size(dtype),
                                    kind == TQ_MEM_HOST ? cudaMemcpyHostToDevice
                                                        : cudaMemcpyDeviceToDevice,
                                    (cudaStream_t)stream);
    // pageable host memory: the copy must finish before the caller may reuse it
    if (e == cudaSuccess && kind == TQ_MEM_HOST) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync");
  }
  if (st == TQ_OK) st = sync_device_meta(t, (cudaStream_t)stream);
  if (st != TQ_OK) {
    tq_bs_destroy(t);
    return st;
  }
  *out = t;
  return TQ_OK;
}

tq_status tq_bs_adopt(tq_dtype dtype, int32_t rank, const int64_t *dimension, int64_t n_blocks,
                      const int64_t *begin_points, const int64_t *end_points,
                      const int64_t *index_tables, const int64_t *block_offsets,
                      void *device_data, tq_bs **out) {
  if (!out) return fail(TQ_ERR_INVALID, "out is NULL");
  if (!device_data) return fail(TQ_ERR_INVALID, "Source data not allocated!");
  if (n_blocks < 0) return fail(TQ_ERR_INVALID, "negative block count");
  if (rank < 0 || rank > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "rank outside 0..12");
  if (rank && !dimension) return fail(TQ_ERR_INVALID, "dimension is NULL");
  if (dtype != TQ_F32 && dtype != TQ_F64 && dtype != TQ_F16)
    return fail(TQ_ERR_INVALID, "unknown dtype");
  if (rank == 0) n_blocks = 0;
  if (n_blocks && (!begin_points || !end_points))
    return fail(TQ_ERR_INVALID, "begin/end points are NULL");
  TQ_CHECK(check_boxes(rank, dimension, n_blocks, begin_points, end_points));
  tq_bs *t = new_tensor(dtype, rank, dimension);
  int64_t added = 0;
  append_meta(t, n_blocks, begin_points, end_points, index_tables, &added);
  if (block_offsets)
    for (int64_t k = 0; k < n_blocks; k++)
      if (block_offsets[k] != t->h_offsets[k]) {
        tq_bs_destroy(t);  // the buffer is still the caller's
        return fail(TQ_ERR_UNSUPPORTED,
                    "block offsets must be the exclusive scan of the block sizes");
      }
  t->data = device_data;
  t->adopted = true;
  t->n_elem = rank == 0 ? 1 : added;
  t->capacity = t->n_elem;
  const tq_status st = sync_device_meta(t, nullptr);
  if (st != TQ_OK) {
    t->data = nullptr;  // a failed adoption leaves the buffer with the caller
    t->adopted = false;
    tq_bs_destroy(t);
    return st;
  }
  *out = t;
  return TQ_OK;
}

tq_status tq_bs_create_zeros(tq_dtype dtype, int32_t rank, const int64_t *dimension,
                             int64_t n_blocks, const int64_t *begin_points,
                             const int64_t *end_points, const int64_t *index_tables,
                             tq_stream stream, tq_bs **out) {
  if (!out) return fail(TQ_ERR_INVALID, "out is NULL");
  if (n_blocks < 0) return fail(TQ_ERR_INVALID, "negative block count");
  if (rank == 0) return tq_bs_create_empty(dtype, 0, nullptr, out);
  if (n_blocks && (!begin_points || !end_points))
    return fail(TQ_ERR_INVALID, "begin/end points are NULL");
  if (rank < 0 || rank > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "rank outside 0..12");
  TQ_CHECK(check_boxes(rank, dimension, n_blocks, begin_points, end_points));
  tq_bs *t = new_tensor(dtype, rank, dimension);
  int64_t added = 0;
  append_meta(t, n_blocks, begin_points, end_points, index_tables, &added);
  tq_status st = alloc_data(t, added, (cudaStream_t)stream);
  if (st == TQ_OK && added) {
    const cudaError_t e = cudaMemsetAsync(t->data, 0, (size_t)added * dtype_size(dtype),
                                          (cudaStream_t)stream);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemsetAsync");
  }
  if (st == TQ_OK) st = sync_device_meta(t, (cudaStream_t)stream);
  if (st != TQ_OK) {
    tq_bs_destroy(t);
    return st;
  }
  *out = t;
  return TQ_OK;
}

tq_status tq_bs_set_data(tq_bs *t, const void *data, tq_memkind kind, tq_stream stream) {
  if (!t) return fail(TQ_ERR_INVALID, "tensor is NULL");
  if (!data) return fail(TQ_ERR_INVALID, "Source data not allocated!");
  const int64_t n = t->rank == 0 ? 1 : t->n_elem;
  if (n == 0) return TQ_OK;
  cudaError_t e = cudaMemcpyAsync(t->data, data, (size_t)n * dtype_size(t->dtype),
                                  kind == TQ_MEM_HOST ? cudaMemcpyHostToDevice
                                                      : cudaMemcpyDeviceToDevice,
                                  (cudaStream_t)stream);
  if (e == cudaSuccess && kind == TQ_MEM_HOST) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
  return TQ_OK;
}

tq_status tq_bs_set_data_async(tq_bs *t, const void *data, tq_memkind kind, tq_stream stream) {
  if (!t) return fail(TQ_ERR_INVALID, "tensor is NULL");
  if (!data) return fail(TQ_ERR_INVALID, "Source data not allocated!");
  if (kind != TQ_MEM_HOST && kind != TQ_MEM_DEVICE) return fail(TQ_ERR_INVALID, "bad memory kind");
  const int64_t n = t->rank == 0 ? 1 : t->n_elem;
  if (n == 0) return TQ_OK;
  TQ_CUDA(cudaMemcpyAsync(t->data, data, (size_t)n * dtype_size(t->dtype),
                          kind == TQ_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                          (cudaStream_t)stream));
  return TQ_OK;
}

tq_status tq_bs_clone(const tq_bs *src, tq_stream stream, tq_bs **out) {
  if (!src || !out) return fail(TQ_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  tq_bs *s_mut = const_cast<tq_bs *>(src);
  TQ_CHECK(sync_host_meta(s_mut, s));
  tq_bs *t = new_tensor(src->dtype, src->rank, src->dimension.data());
  t->nb = src->nb;
  t->h_begin = src->h_begin;
  t->h_end = src->h_end;
  t->h_strides = src->h_strides;
  t->h_offsets = src->h_offsets;
  tq_status st = alloc_data(t, src->n_elem, s);
  if (st == TQ_OK) {
    size_t bytes = (size_t)(src->rank == 0 ? 1 : src->n_elem) * dtype_size(src->dtype);
    cudaError_t e = bytes ? cudaMemcpyAsync(t->data, src->data, bytes, cudaMemcpyDeviceToDevice, s)
                          : cudaSuccess;
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync");
  }
  if (st == TQ_OK) st = sync_device_meta(t, s);
  if (st != TQ_OK) {
    tq_bs_destroy(t);
    return st;
  }
  *out = t;
  return TQ_OK;
}

tq_status tq_bs_destroy(tq_bs *t) {
  if (!t) return TQ_OK;
  free_data(t);
  t->d_meta.release();
  delete t;
  return TQ_OK;
}

tq_status tq_bs_append_blocks(tq_bs *t, int64_t n, const int64_t *b, const int64_t *e,
                              const int64_t *tables, const void *data, tq_memkind kind,
                              tq_stream stream) {
  if (!t) return fail(TQ_ERR_INVALID, "tensor is NULL");
  if (n < 0) return fail(TQ_ERR_INVALID, "negative block count");
  if (n == 0) return TQ_OK;
  if (t->rank == 0) return fail(TQ_ERR_INVALID, "cannot append blocks to a rank-0 tensor");
  if (!b || !e || !data) return fail(TQ_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CHECK(sync_host_meta(t, s));
  TQ_CHECK(check_boxes(t->rank, t->dimension.data(), n, b, e));
  const int64_t old = t->n_elem;
  int64_t added = 0;
  // compute the new element count first so a failed allocation leaves t intact
  {
    int64_t total = 0;
    for (int64_t k = 0; k < n; k++) {
      int64_t cnt = 1;
      for (int32_t l = 0; l < t->rank; l++) cnt *= e[k * t->rank + l] - b[k * t->rank + l] + 1;
      total += cnt;
    }
    added = total;
  }
  if (old + added > t->capacity) {
    int64_t cap = t->capacity * 2;
    if (cap < old + added) cap = old + added;
    void *nd = nullptr;
    TQ_CHECK(dev_alloc(&nd, (size_t)cap * dtype_size(t->dtype), s));
    if (old) {
      cudaError_t err = cudaMemcpyAsync(nd, t->data, (size_t)old * dtype_size(t->dtype),
                                        cudaMemcpyDeviceToDevice, s);
      if (err != cudaSuccess) {
        dev_free(nd, s);
        return cuda_fail(err, "cudaMemcpyAsync");
      }
    }
    free_data(t);
    t->data = nd;
    t->alloc_stream = s;
    t->capacity = cap;
  }
  int64_t chk = 0;
  append_meta(t, n, b, e, tables, &chk);
  t->n_elem = old + added;
  TQ_CUDA(cudaMemcpyAsync((char *)t->data + (size_t)old * dtype_size(t->dtype), data,
                          (size_t)added * dtype_size(t->dtype),
                          kind == TQ_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                          s));
  if (kind == TQ_MEM_HOST) TQ_CUDA(cudaStreamSynchronize(s));
  return sync_device_meta(t, s);
}

static tq_status check_index(const tq_bs *t, const int64_t *idx) {
  for (int32_t l = 0; l < t->rank; l++)
    if (idx[l] < 0 || idx[l] >= t->dimension[l])
      return fail(TQ_ERR_RANGE, "Indices out of boundary");
  return TQ_OK;
}

static void blocks_holding(const tq_bs *t, const int64_t *idx, std::vector<int64_t> &hits) {
  for (int64_t k = 0; k < t->nb; k++) {
    bool in = true;
    for (int32_t l = 0; l < t->rank && in; l++)
      in = idx[l] >= t->h_begin[k * t->rank + l] && idx[l] <= t->h_end[k * t->rank + l];
    if (in) hits.push_back(k);
  }
}

static int64_t element_address(const tq_bs *t, int64_t k, const int64_t *idx) {
  int64_t a = t->h_offsets[k];
  for (int32_t l = 0; l < t->rank; l++)
    a += (idx[l] - t->h_begin[k * t->rank + l]) * t->h_strides[k * t->rank + l];
  return a;
}

tq_status tq_bs_query(const tq_bs *t, const int64_t *idx, void *value) {
  if (!t || !value) return fail(TQ_ERR_INVALID, "NULL argument");
  if (t->rank && !idx) return fail(TQ_ERR_INVALID, "indices are NULL");
  TQ_CHECK(check_index(t, idx));
  tq_bs *tm = const_cast<tq_bs *>(t);
  TQ_CHECK(sync_host_meta(tm, nullptr));
  TQ_CUDA(cudaDeviceSynchronize());
  const size_t es = dtype_size(t->dtype);
  if (t->rank == 0) {
    TQ_CUDA(cudaMemcpy(value, t->data, es, cudaMemcpyDeviceToHost));
    return TQ_OK;
  }
  std::vector<int64_t> hits;
  blocks_holding(t, idx, hits);
  double acc = 0.0;
  float accf = 0.0f;
  for (int64_t k : hits) {
    const int64_t a = element_address(t, k, idx);
    if (t->dtype == TQ_F64) {
      double v;
      TQ_CUDA(cudaMemcpy(&v, (const double *)t->data + a, 8, cudaMemcpyDeviceToHost));
      acc += v;
    } else if (t->dtype == TQ_F32) {
      float v;
      TQ_CUDA(cudaMemcpy(&v, (const float *)t->data + a, 4, cudaMemcpyDeviceToHost));
      accf += v;
    } else {
      __half v;
      TQ_CUDA(cudaMemcpy(&v, (const __half *)t->data + a, 2, cudaMemcpyDeviceToHost));
      accf += __half2float(v);
    }
  }
  if (t->dtype == TQ_F64) {
    std::memcpy(value, &acc, 8);
  } else if (t->dtype == TQ_F32) {
    std::memcpy(value, &accf, 4);
  } else {
    const __half h = __float2half_rn(accf);
    std::memcpy(value, &h, 2);
  }
  return TQ_OK;
}

tq_status tq_bs_modify(tq_bs *t, const int64_t *idx, const void *value) {
  if (!t || !value) return fail(TQ_ERR_INVALID, "NULL argument");
  if (t->rank && !idx) return fail(TQ_ERR_INVALID, "indices are NULL");
  TQ_CHECK(check_index(t, idx));
  TQ_CHECK(sync_host_meta(t, nullptr));
  TQ_CUDA(cudaDeviceSynchronize());
  const size_t es = dtype_size(t->dtype);
  if (t->rank == 0) {
    TQ_CUDA(cudaMemcpy(t->data, value, es, cudaMemcpyHostToDevice));
    return TQ_OK;
  }
  std::vector<int64_t> hits;
  blocks_holding(t, idx, hits);
  if (!hits.empty()) {
    TQ_CUDA(cudaMemcpy((char *)t->data + element_address(t, hits[0], idx) * es, value, es,
                       cudaMemcpyHostToDevice));
    for (size_t q = 1; q < hits.size(); q++)
      TQ_CUDA(cudaMemset((char *)t->data + element_address(t, hits[q], idx) * es, 0, es));
    return TQ_OK;
  }
  const bool nonzero = t->dtype == TQ_F64   ? *(const double *)value != 0.0
                       : t->dtype == TQ_F32 ? *(const float *)value != 0.0f
                                            : __half2float(*(const __half *)value) != 0.0f;
  if (!nonzero) return TQ_OK;
  // a one-element block with an all-zero index table, as the reference appends
  std::vector<int64_t> zeros(t->rank, 0);
  return tq_bs_append_blocks(t, 1, idx, idx, zeros.data(), value, TQ_MEM_HOST, nullptr);
}

tq_status tq_bs_to_number(const tq_bs *t, void *value) {
  if (!t || !value) return fail(TQ_ERR_INVALID, "NULL argument");
  if (t->rank != 0) return fail(TQ_ERR_INVALID, "to_number needs a rank-0 tensor");
  TQ_CUDA(cudaDeviceSynchronize());
  TQ_CUDA(cudaMemcpy(value, t->data, dtype_size(t->dtype), cudaMemcpyDeviceToHost));
  return TQ_OK;
}

tq_status tq_bs_shape(const tq_bs *t, tq_dtype *dtype, int32_t *rank, int64_t *n_blocks,
                      int64_t *n_elem) {
  if (!t) return fail(TQ_ERR_INVALID, "tensor is NULL");
  if (dtype) *dtype = t->dtype;
  if (rank) *rank = t->rank;
  if (n_blocks) *n_blocks = t->nb;
  if (n_elem) *n_elem = t->n_elem;
  return TQ_OK;
}

tq_status tq_bs_metadata(const tq_bs *t, int64_t *dimension, int64_t *begin, int64_t *end,
                         int64_t *tables, int64_t *offsets) {
  if (!t) return fail(TQ_ERR_INVALID, "tensor is NULL");
  tq_bs *tm = const_cast<tq_bs *>(t);
  TQ_CHECK(sync_host_meta(tm, nullptr));
  const size_t nr = (size_t)t->nb * t->rank;
  if (dimension && t->rank) std::memcpy(dimension, t->dimension.data(), t->rank * 8);
  if (begin && nr) std::memcpy(begin, t->h_begin.data(), nr * 8);
  if (end && nr) std::memcpy(end, t->h_end.data(), nr * 8);
  if (tables && nr) std::memcpy(tables, t->h_strides.data(), nr * 8);
  if (offsets && t->nb) std::memcpy(offsets, t->h_offsets.data(), t->nb * 8);
  return TQ_OK;
}

tq_status tq_bs_device_data(const tq_bs *t, void **ptr) {
  if (!t || !ptr) return fail(TQ_ERR_INVALID, "NULL argument");
  *ptr = t->data;
  return TQ_OK;
}

tq_status tq_bs_copy_data(const tq_bs *t, void *dst, tq_memkind kind, tq_stream stream) {
  if (!t || !dst) return fail(TQ_ERR_INVALID, "NULL argument");
  const size_t bytes = (size_t)(t->rank == 0 ? 1 : t->n_elem) * dtype_size(t->dtype);
  if (!bytes) return TQ_OK;
  TQ_CUDA(cudaMemcpyAsync(dst, t->data, bytes,
                          kind == TQ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                          (cudaStream_t)stream));
  if (kind == TQ_MEM_HOST) TQ_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return TQ_OK;
}

tq_status tq_bs_slice(const tq_bs *src, const int64_t *divisor, tq_stream stream, tq_bs **out) {
  // Splits every block into prod(divisor) boxes; the data are copied as they
  // are, so values are reinterpreted exactly as in block_sparse.cuh:1124-1176.
  if (!src || !divisor || !out) return fail(TQ_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  tq_bs *sm = const_cast<tq_bs *>(src);
  TQ_CHECK(sync_host_meta(sm, s));
  const int32_t r = src->rank;
  int64_t nsub = 1;
  for (int32_t l = 0; l < r; l++) {
    if (divisor[l] <= 0) return fail(TQ_ERR_INVALID, "divisor must be positive");
    nsub *= divisor[l];
  }
  std::vector<int64_t> nb_, ne_, nt_;
  for (int64_t k = 0; k < src->nb; k++) {
    int64_t sub[TQ_MAXR];
    for (int32_t l = 0; l < r; l++) {
      const int64_t d = src->h_end[k * r + l] - src->h_begin[k * r + l] + 1;
      if (d % divisor[l]) return fail(TQ_ERR_INVALID, "current slice does not support residues");
      sub[l] = d / divisor[l];
    }
    for (int64_t q = 0; q < nsub; q++) {
      int64_t t = q;
      for (int32_t l = 0; l < r; l++) {
        const int64_t x = t % divisor[l];
        t /= divisor[l];
        const int64_t b0 = src->h_begin[k * r + l] + x * sub[l];
        nb_.push_back(b0);
        ne_.push_back(b0 + sub[l] - 1);
      }
    }
  }
  // The reference re-derives column-major index tables in the constructor it
  // calls (block_sparse.cuh:1173-1174), so the computed tables are not used.
  return tq_bs_create(src->dtype, r, src->dimension.data(), src->nb * nsub, nb_.data(),
                      ne_.data(), nullptr, src->data, TQ_MEM_DEVICE, stream, out);
}

}  // extern "C"
