// hard_transpose: permute the legs of every block
// (src/gpu/block_sparse.cuh:1031-1122; CPU semantics src/tensor/block_sparse.h:608-651).
//
// The reference packs all blocks into a stack padded to the global maximum
// block dims, permutes it with cuTT and unpacks it (memory = max dims x
// n_blocks).  Here every block is permuted in place of its own extent.  The
// unit of work is the "plane" of input leg 0 and the leg that becomes output
// leg 0 (p0), for one combination of the other legs: contiguous in the input
// along leg 0 and in the output along leg p0.  Sector-sized blocks have small
// planes, so a tile batches up to 256 planes of up to PLANE_MAX elements: the
// planes' base offsets are decoded once per plane into shared memory, the
// elements are read along input leg 0 into a padded shared buffer and written
// along output leg 0.  When leg 0 stays leg 0 a plane is a contiguous run and
// is copied straight.  Planes too large for the buffer fall back to 32 x 32
// tiles.  Tiles are walked by a persistent grid; one load finds a tile's block.
#include <cstring>

#include "index.cuh"
#include "tq_internal.h"

namespace tq {

constexpr int TT = 32;            // edge of the large-plane tiles
constexpr int PLANE_MAX = 4096;   // elements of the shared buffer
constexpr int PLANES_MAX = 256;   // planes per tile

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

// Tiling of one block (host and device agree through this one function).
// mode 0: runs (p0 == 0), 1: batched planes, 2: 32 x 32 tiles.
struct PlanePlan {
  int mode;
  uint32_t P;        // elements of a plane in the shared buffer (padded, mode 1)
  uint32_t ppc;      // planes per tile (modes 0 and 1)
  uint32_t rows;     // planes of the block (product of the other legs)
  int64_t tiles;
};

__host__ __device__ inline PlanePlan plane_plan(const uint32_t *d, int r, int p0) {
  PlanePlan pp;
  uint64_t rows = 1;
  for (int l = 1; l < r; l++)
    if (l != p0) rows *= d[l];
  pp.rows = (uint32_t)rows;
  if (p0 == 0) {
    pp.mode = 0;
    pp.P = d[0];
    uint32_t ppc = PLANE_MAX / (d[0] ? d[0] : 1);
    ppc = ppc < 1 ? 1 : (ppc > PLANES_MAX ? PLANES_MAX : ppc);
    pp.ppc = ppc;
    pp.tiles = d[0] > (uint32_t)PLANE_MAX ? (int64_t)rows * ((d[0] + PLANE_MAX - 1) / PLANE_MAX)
                                          : (int64_t)((rows + ppc - 1) / ppc);
    return pp;
  }
  const uint64_t P = (uint64_t)(d[0] + 1) * d[p0];  // leg-0 runs padded by one
  if (P <= (uint64_t)PLANE_MAX) {
    pp.mode = 1;
    pp.P = (uint32_t)P;
    uint32_t ppc = PLANE_MAX / pp.P;
    pp.ppc = ppc > PLANES_MAX ? PLANES_MAX : ppc;
    pp.tiles = (int64_t)((rows + pp.ppc - 1) / pp.ppc);
    return pp;
  }
  pp.mode = 2;
  pp.P = 0;
  pp.ppc = 1;
  pp.tiles = (int64_t)((d[0] + TT - 1) / TT) * ((d[p0] + TT - 1) / TT) * (int64_t)rows;
  return pp;
}

// block of every tile (one load per tile instead of a search)
__global__ void tile_block_kernel(const int64_t *tile_start, int64_t nb, int64_t n_tiles,
                                  int32_t *tile_block) {
  const int64_t b = (int64_t)blockIdx.x;
  if (b >= nb) return;
  const int64_t t0 = tile_start[b], t1 = b + 1 < nb ? tile_start[b + 1] : n_tiles;
  for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) tile_block[t] = (int32_t)b;
}

// Offsets in the input and the output of plane `row` (the other legs in input
// order, lowest leg fastest).
__device__ __forceinline__ void plane_bases(uint32_t row, const uint32_t *d, const int64_t *st,
                                            const int64_t *ost, int r, int p0, int64_t &ib,
                                            int64_t &ob) {
  for (int l = 1; l < r; l++) {
    if (l == p0) continue;
    const uint32_t c = row % d[l];
    row /= d[l];
    ib += c * st[l];
    ob += c * ost[l];
  }
}

// x / d for x < 8192 and 1 <= d <= 4096 by a multiply with m = 2^32 / d
// rounded up (exact over that range: checked for every x and d), d = 1 apart.
struct SmallDiv {
  uint32_t d, m;
  __device__ __forceinline__ explicit SmallDiv(uint32_t dd)
      : d(dd), m(dd > 1 ? 0xFFFFFFFFu / dd + 1u : 0u) {}
  __device__ __forceinline__ uint32_t div(uint32_t x) const { return d > 1 ? __umulhi(x, m) : x; }
};

template <typename T>
__global__ void __launch_bounds__(256) transpose_kernel(TransposeJob job, int64_t n_tiles) {
  __shared__ T buf[PLANE_MAX];
  __shared__ int64_t base_in[PLANES_MAX], base_out[PLANES_MAX];
  const int r = job.rank;
  const int p0 = job.perm[0];
  const T *__restrict__ src = (const T *)job.in.data;
  T *__restrict__ dst = (T *)job.out;
  const int tid = threadIdx.x;
  for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const int64_t b = job.tile_block[t];
    const uint32_t local = (uint32_t)(t - job.tile_start[b]);
    const int64_t *bb = job.in.begin + b * r, *be = job.in.end + b * r;
    const int64_t *st = job.in.strides + b * r;
    uint32_t d[TQ_MAXR];
    for (int l = 0; l < r; l++) d[l] = (uint32_t)(be[l] - bb[l] + 1);
    int64_t ost[TQ_MAXR];  // stride in the output of INPUT leg l
    {
      int64_t sacc = 1;
      for (int q = 0; q < r; q++) {
        ost[job.perm[q]] = sacc;
        sacc *= d[job.perm[q]];
      }
    }
    const PlanePlan pp = plane_plan(d, r, p0);
    const int64_t ib0 = job.in.offsets[b], ob0 = job.out_off[b];
    // the strides the element loops use, in registers: read through pointers
    // they would be reloaded after every store (the stores might alias them)
    const int64_t s0 = st[0], sp = st[p0], o0 = ost[0], op = ost[p0];
    __syncthreads();  // the previous tile is done with the shared arrays
    if (pp.mode == 2) {
      // one 32 x 32 tile of a large plane
      const uint32_t n0 = (d[0] + TT - 1) / TT, np = (d[p0] + TT - 1) / TT;
      const uint32_t i0 = (local % n0) * TT, j0 = ((local / n0) % np) * TT;
      int64_t ib = ib0, ob = ob0;
      plane_bases(local / n0 / np, d, st, ost, r, p0, ib, ob);
      T(*tile)[TT + 1] = reinterpret_cast<T(*)[TT + 1]>(buf);
      const int tx = tid & 31, ty = tid >> 5;
      for (int q = ty; q < TT; q += 8) {
        const uint32_t ii = i0 + tx, jj = j0 + q;
        if (ii < d[0] && jj < d[p0]) tile[q][tx] = src[ib + ii * s0 + jj * sp];
      }
      __syncthreads();
      for (int q = ty; q < TT; q += 8) {
        const uint32_t jj = j0 + tx, ii = i0 + q;
        if (ii < d[0] && jj < d[p0]) dst[ob + jj * op + ii * o0] = tile[tx][q];
      }
      continue;
    }
    if (pp.mode == 0 && d[0] > (uint32_t)PLANE_MAX) {
      // one PLANE_MAX-long piece of a long run
      const uint32_t npc = (d[0] + PLANE_MAX - 1) / PLANE_MAX;
      const uint32_t i0 = (local % npc) * PLANE_MAX;
      int64_t ib = ib0, ob = ob0;
      plane_bases(local / npc, d, st, ost, r, p0, ib, ob);
      for (uint32_t i = i0 + tid; i < d[0] && i < i0 + PLANE_MAX; i += 256)
        dst[ob + i * o0] = src[ib + i * s0];
      continue;
    }
    // batched planes: bases first, one thread per plane
    const uint32_t row0 = local * pp.ppc;
    const uint32_t nrows = pp.rows - row0 < pp.ppc ? pp.rows - row0 : pp.ppc;
    if ((uint32_t)tid < nrows) {
      int64_t ib = ib0, ob = ob0;
      plane_bases(row0 + tid, d, st, ost, r, p0, ib, ob);
      base_in[tid] = ib;
      base_out[tid] = ob;
    }
    __syncthreads();
    if (pp.mode == 0) {
      // nrows * d0 <= PLANE_MAX here
      const SmallDiv by_d0(d[0]);
      const uint32_t n = nrows * d[0];
      for (uint32_t e = tid; e < n; e += 256) {
        const uint32_t pi = by_d0.div(e), i = e - pi * d[0];
        dst[base_out[pi] + i * o0] = src[base_in[pi] + i * s0];
      }
      continue;
    }
    // mode 1: plane pi sits at buf[pi * P + i + j * (d0 + 1)]; n <= PLANE_MAX
    const uint32_t d0 = d[0], dp = d[p0], PL = d0 * dp, n = nrows * PL;
    const SmallDiv by_pl(PL), by_d0(d0), by_dp(dp);
    for (uint32_t e = tid; e < n; e += 256) {
      const uint32_t pi = by_pl.div(e), w = e - pi * PL, j = by_d0.div(w), i = w - j * d0;
      buf[pi * pp.P + i + j * (d0 + 1)] = src[base_in[pi] + i * s0 + j * sp];
    }
    __syncthreads();
    for (uint32_t f = tid; f < n; f += 256) {
      const uint32_t pi = by_pl.div(f), w = f - pi * PL, i = by_dp.div(w), j = w - i * dp;
      dst[base_out[pi] + j * op + i * o0] = buf[pi * pp.P + i + j * (d0 + 1)];
    }
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
    // tiles per block from the host metadata (no device round trip)
    const int32_t p0 = (int32_t)perm[0];
    std::vector<int64_t> h_start(t->nb);
    int64_t n_tiles = 0;
    for (int64_t b = 0; b < t->nb; b++) {
      uint32_t d[TQ_MAXR];
      uint64_t prod = 1;
      for (int32_t l = 0; l < r; l++) {
        const int64_t x = t->h_end[b * r + l] - t->h_begin[b * r + l] + 1;
        prod *= (uint64_t)x;
        if (x >= (int64_t(1) << 31) || prod >= (uint64_t(1) << 31))
          return fail(TQ_ERR_UNSUPPORTED, "a block of 2^31 elements or more");
        d[l] = (uint32_t)x;
      }
      h_start[b] = n_tiles;
      n_tiles += plane_plan(d, r, p0).tiles;
    }
    if (n_tiles > 0x7fffffffLL) return fail(TQ_ERR_UNSUPPORTED, "more than 2^31 transpose tiles");
    if (t->nb > 0x7fffffffLL) return fail(TQ_ERR_UNSUPPORTED, "more than 2^31 blocks");
    DevArray<int64_t> tile_start;
    DevArray<int32_t> tile_block;
    TQ_CHECK(tile_start.alloc(t->nb, s));
    TQ_CHECK(tile_block.alloc(std::max<int64_t>(n_tiles, 1), s));
    TQ_CUDA(cudaMemcpyAsync(tile_start.p, h_start.data(), t->nb * 8, cudaMemcpyHostToDevice, s));
    TQ_CUDA(cudaStreamSynchronize(s));  // h_start dies with this function
    TransposeJob job;
    job.in = t->view();
    job.rank = r;
    for (int32_t l = 0; l < r; l++) job.perm[l] = (int32_t)perm[l];
    job.out_off = o->d_meta.p + 3 * o->nb * r;
    job.tile_start = tile_start.p;
    job.tile_block = tile_block.p;
    job.nb = t->nb;
    job.out = o->data;
    if (n_tiles) {
      count_launch(), tile_block_kernel<<<(unsigned)t->nb, 256, 0, s>>>(tile_start.p, t->nb, n_tiles,
                                                                         tile_block.p);
      int dev = 0, sms = 0;
      TQ_CUDA(cudaGetDevice(&dev));
      TQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      const unsigned grid = (unsigned)std::min<int64_t>(n_tiles, 6 * (int64_t)sms);
      // a transpose moves bits: the element size picks the kernel
      if (t->dtype == TQ_F64)
        count_launch(), transpose_kernel<double><<<grid, 256, 0, s>>>(job, n_tiles);
      else if (t->dtype == TQ_F32)
        count_launch(), transpose_kernel<float><<<grid, 256, 0, s>>>(job, n_tiles);
      else
        count_launch(), transpose_kernel<unsigned short><<<grid, 256, 0, s>>>(job, n_tiles);
      TQ_CUDA(cudaGetLastError());
    }
  }
  *out = guard.release();
  return TQ_OK;
}
