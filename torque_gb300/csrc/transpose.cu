// hard_transpose: permute the legs of every block
// (src/gpu/block_sparse.cuh:1031-1122; CPU semantics src/tensor/block_sparse.h:608-651).
//
// The reference packs all blocks into a stack padded to the global maximum
// block dims, permutes it with cuTT and unpacks it (memory = max dims x
// n_blocks).  Here every block is permuted in place of its own extent: a work
// list of 32x32 tiles spanning (input leg 0) x (output leg 0), batched over the
// other legs, staged through shared memory so that both the reads and the
// writes run along the unit-stride leg.  When leg 0 stays leg 0 the tile is a
// straight copy of contiguous runs.
#include <cstring>

#include "index.cuh"
#include "tq_internal.h"

namespace tq {

constexpr int TT = 32;  // tile edge

struct TransposeJob {
  DevBS in;
  int32_t rank;
  int32_t perm[TQ_MAXR];
  const int64_t *out_off;     // output block offsets
  const int64_t *tile_start;  // [nb+1]
  int64_t nb;
  void *out;
};

__device__ __forceinline__ int64_t find_block(const int64_t *start, int64_t n, int64_t t) {
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (start[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Tiles of block b: ceil(d_in0/32) * ceil(d_out0/32) * prod(other dims), where
// d_in0 = dim of input leg 0 and d_out0 = dim of input leg perm[0].
__global__ void transpose_tiles_kernel(DevBS in, int32_t p0, int64_t *tiles) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= in.nb) return;
  const int64_t *bb = in.begin + b * in.rank, *be = in.end + b * in.rank;
  int64_t n = 1;
  for (int l = 0; l < in.rank; l++) {
    const int64_t d = be[l] - bb[l] + 1;
    if (l == 0 || l == p0) n *= (d + TT - 1) / TT;
    else n *= d;
  }
  tiles[b] = in.rank ? n : 0;
}

template <typename T>
__global__ void __launch_bounds__(256) transpose_kernel(TransposeJob job) {
  __shared__ T tile[TT][TT + 1];
  __shared__ int64_t s_b, s_local;
  const int64_t t = blockIdx.x;
  if (threadIdx.x == 0) {
    s_b = find_block(job.tile_start, job.nb, t);
    s_local = t - job.tile_start[s_b];
  }
  __syncthreads();
  const int64_t b = s_b;
  const int r = job.rank;
  const int32_t p0 = job.perm[0];
  const int64_t *bb = job.in.begin + b * r, *be = job.in.end + b * r;
  const int64_t *st = job.in.strides + b * r;
  int64_t d[TQ_MAXR];
  for (int l = 0; l < r; l++) d[l] = be[l] - bb[l] + 1;
  // output strides: column-major over the permuted dims
  int64_t ost[TQ_MAXR];  // stride in the output of INPUT leg l
  {
    int64_t s = 1;
    for (int q = 0; q < r; q++) {
      ost[job.perm[q]] = s;
      s *= d[job.perm[q]];
    }
  }
  // decode the tile: leg 0 tile, leg p0 tile, then the other legs
  int64_t x = s_local;
  const int64_t n0 = (d[0] + TT - 1) / TT;
  const int64_t i0 = (x % n0) * TT;
  x /= n0;
  int64_t j0 = 0;
  if (p0 != 0) {
    const int64_t np = (d[p0] + TT - 1) / TT;
    j0 = (x % np) * TT;
    x /= np;
  }
  int64_t in_base = job.in.offsets[b], out_base = job.out_off[b];
  for (int l = 1; l < r; l++) {
    if (l == p0) continue;
    const int64_t c = x % d[l];
    x /= d[l];
    in_base += c * st[l];
    out_base += c * ost[l];
  }
  const T *src = (const T *)job.in.data;
  T *dst = (T *)job.out;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  if (p0 == 0) {
    // leg 0 stays fastest: copy up to 32 contiguous elements of leg 0
    if (ty == 0 && i0 + tx < d[0])
      dst[out_base + (i0 + tx) * ost[0]] = src[in_base + (i0 + tx) * st[0]];
    return;
  }
  // read along input leg 0, write along output leg 0 (= input leg p0)
  for (int q = ty; q < TT; q += 8) {
    const int64_t ii = i0 + tx, jj = j0 + q;
    if (ii < d[0] && jj < d[p0]) tile[q][tx] = src[in_base + ii * st[0] + jj * st[p0]];
  }
  __syncthreads();
  for (int q = ty; q < TT; q += 8) {
    const int64_t jj = j0 + tx, ii = i0 + q;
    if (ii < d[0] && jj < d[p0]) dst[out_base + jj * ost[p0] + ii * ost[0]] = tile[tx][q];
  }
}

}  // namespace tq

using namespace tq;

extern "C" tq_status tq_bs_hard_transpose(const tq_bs *t, const int64_t *perm, tq_stream stream,
                                          tq_bs **out) {
  if (!t || !out) return fail(TQ_ERR_INVALID, "NULL argument");
  if (t->rank && !perm) return fail(TQ_ERR_INVALID, "perm is NULL");
  bool seen[TQ_MAXR] = {false};
  for (int32_t l = 0; l < t->rank; l++) {
    if (perm[l] < 0 || perm[l] >= t->rank || seen[perm[l]])
      return fail(TQ_ERR_INVALID, "The number of permutation does not match the rank of tensor");
    seen[perm[l]] = true;
  }
  cudaStream_t s = (cudaStream_t)stream;
  tq_bs *tm = const_cast<tq_bs *>(t);
  TQ_CHECK(sync_host_meta(tm, s));
  TQ_CHECK(sync_device_meta(tm, s));
  const int32_t r = t->rank;
  std::vector<int64_t> nd(r), nb_(t->nb * r), ne_(t->nb * r);
  for (int32_t l = 0; l < r; l++) nd[l] = t->dimension[perm[l]];
  for (int64_t b = 0; b < t->nb; b++)
    for (int32_t l = 0; l < r; l++) {
      nb_[b * r + l] = t->h_begin[b * r + perm[l]];
      ne_[b * r + l] = t->h_end[b * r + perm[l]];
    }
  tq_bs *o = new_tensor(t->dtype, r, nd.data());
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> guard(o, tq_bs_destroy);
  if (r == 0) {
    TQ_CHECK(alloc_data(o, 1, s));
    TQ_CUDA(cudaMemcpyAsync(o->data, t->data, dtype_size(t->dtype), cudaMemcpyDeviceToDevice, s));
    *out = guard.release();
    return TQ_OK;
  }
  o->nb = t->nb;
  o->h_begin = nb_;
  o->h_end = ne_;
  o->h_strides.resize(t->nb * r);
  o->h_offsets.resize(t->nb);
  int64_t off = 0;
  for (int64_t b = 0; b < t->nb; b++) {
    int64_t s1 = 1;
    for (int32_t l = 0; l < r; l++) {
      o->h_strides[b * r + l] = s1;
      s1 *= ne_[b * r + l] - nb_[b * r + l] + 1;
    }
    o->h_offsets[b] = off;
    off += s1;
  }
  TQ_CHECK(alloc_data(o, off, s));
  TQ_CHECK(sync_device_meta(o, s));
  if (t->nb) {
    DevArray<int64_t> tiles, tile_start, total;
    TQ_CHECK(tiles.alloc(t->nb, s));
    TQ_CHECK(tile_start.alloc(t->nb, s));
    TQ_CHECK(total.alloc(1, s));
    const DevBS v = t->view();
    count_launch(), transpose_tiles_kernel<<<(unsigned)((t->nb + 255) / 256), 256, 0, s>>>(v, (int32_t)perm[0],
                                                                         tiles.p);
    TQ_CHECK(scan_exclusive(tiles.p, tile_start.p, t->nb, total.p, s));
    int64_t n_tiles = 0;
    TQ_CUDA(cudaMemcpyAsync(&n_tiles, total.p, 8, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaStreamSynchronize(s));
    TransposeJob job;
    job.in = v;
    job.rank = r;
    for (int32_t l = 0; l < r; l++) job.perm[l] = (int32_t)perm[l];
    job.out_off = o->d_meta.p + 3 * o->nb * r;
    job.tile_start = tile_start.p;
    job.nb = t->nb;
    job.out = o->data;
    if (n_tiles > 0x7fffffffLL) return fail(TQ_ERR_UNSUPPORTED, "more than 2^31 transpose tiles");
    if (n_tiles) {
      if (t->dtype == TQ_F64)
        count_launch(), transpose_kernel<double><<<(unsigned)n_tiles, 256, 0, s>>>(job);
      else
        count_launch(), transpose_kernel<float><<<(unsigned)n_tiles, 256, 0, s>>>(job);
      TQ_CUDA(cudaGetLastError());
    }
  }
  *out = guard.release();
  return TQ_OK;
}
