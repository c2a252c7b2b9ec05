// hard_transpose: permute the legs of every block
// (src/gpu/block_sparse.cuh:1031-1122; CPU semantics src/tensor/block_sparse.h:608-651).
//
// The reference packs all blocks into a stack padded to the global maximum
// block dims, permutes it with cuTT and unpacks it (memory = max dims x
// n_blocks).  Here every block is permuted in place of its own extent: a work
// list of 32x32 tiles spanning (input leg 0) x (output leg 0), batched over the
// other legs, staged through shared memory so that both the reads and the
// writes run along the unit-stride leg.  When leg 0 stays leg 0 a tile is 8
// straight copies of contiguous runs, one per warp.
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
  const int64_t *tile_start;  // [nb] first tile of each block
  const int32_t *tile_block;  // [n_tiles] block of each tile
  int64_t nb;
  void *out;
};

// Tiles of block b.  Transposing (leg 0 moves): ceil(d_in0/32) * ceil(d_out0/32)
// * prod(other dims), d_out0 = dim of input leg perm[0], 32x32 tiles through
// shared memory.  Leg 0 stays: ceil(d_0/32) * ceil(prod(other dims)/8), each
// tile 8 runs of up to 32 contiguous elements (one warp per run).
__global__ void transpose_tiles_kernel(DevBS in, int32_t p0, int64_t *tiles) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= in.nb) return;
  const int64_t *bb = in.begin + b * in.rank, *be = in.end + b * in.rank;
  int64_t n = 1, rest = 1;
  for (int l = 0; l < in.rank; l++) {
    const int64_t d = be[l] - bb[l] + 1;
    if (l == 0 || l == p0) n *= (d + TT - 1) / TT;
    else rest *= d;
  }
  tiles[b] = !in.rank ? 0 : p0 == 0 ? n * ((rest + 7) / 8) : n * rest;
}

// block of every tile (one load per CTA instead of a search)
__global__ void tile_block_kernel(const int64_t *tile_start, int64_t nb, int64_t n_tiles,
                                  int32_t *tile_block) {
  const int64_t b = (int64_t)blockIdx.x;
  if (b >= nb) return;
  const int64_t t0 = tile_start[b], t1 = b + 1 < nb ? tile_start[b + 1] : n_tiles;
  for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) tile_block[t] = (int32_t)b;
}

template <typename T>
__global__ void __launch_bounds__(256) transpose_kernel(TransposeJob job) {
  __shared__ T tile[TT][TT + 1];
  const int64_t t = blockIdx.x;
  const int64_t b = job.tile_block[t];
  const int64_t local = t - job.tile_start[b];
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
  const T *src = (const T *)job.in.data;
  T *dst = (T *)job.out;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int64_t n0 = (d[0] + TT - 1) / TT;
  const int64_t i0 = (local % n0) * TT;
  int64_t x = local / n0;
  if (p0 == 0) {
    // leg 0 stays fastest: warp ty copies the run of row 8*x + ty (the other
    // legs in input order, leg 1 fastest), up to 32 elements of leg 0
    int64_t row = 8 * x + ty, in_base = job.in.offsets[b], out_base = job.out_off[b];
    for (int l = 1; l < r; l++) {
      const int64_t c = row % d[l];
      row /= d[l];
      in_base += c * st[l];
      out_base += c * ost[l];
    }
    if (row == 0 && i0 + tx < d[0])
      dst[out_base + (i0 + tx) * ost[0]] = src[in_base + (i0 + tx) * st[0]];
    return;
  }
  // decode the rest of the tile: leg p0 tile, then the other legs
  const int64_t np = (d[p0] + TT - 1) / TT;
  const int64_t j0 = (x % np) * TT;
  x /= np;
  int64_t in_base = job.in.offsets[b], out_base = job.out_off[b];
  for (int l = 1; l < r; l++) {
    if (l == p0) continue;
    const int64_t c = x % d[l];
    x /= d[l];
    in_base += c * st[l];
    out_base += c * ost[l];
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
    DevArray<int32_t> tile_block;
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
    if (t->nb > 0x7fffffffLL) return fail(TQ_ERR_UNSUPPORTED, "more than 2^31 blocks");
    TQ_CHECK(tile_block.alloc(std::max<int64_t>(n_tiles, 1), s));
    job.tile_block = tile_block.p;
    if (n_tiles) {
      count_launch(), tile_block_kernel<<<(unsigned)t->nb, 256, 0, s>>>(tile_start.p, t->nb, n_tiles,
                                                                         tile_block.p);
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
