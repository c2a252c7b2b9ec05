// Integer index kernels: prefix scans, a stable radix sort and block-pair
// matching.  Integer work only; every result is bit-exact and independent of
// scheduling (no atomics decide an order).
#include <mutex>

#include "index.cuh"

namespace tq {

// ---------------------------------------------------------------- scan
// Three-phase tiled scan: tile sums, scan of the sums (recursive), rescan with
// the tile offset.  Tile = 256 threads x 8 consecutive elements.
constexpr int SCAN_T = 256, SCAN_V = 8, SCAN_TILE = SCAN_T * SCAN_V;

__device__ __forceinline__ int64_t block_exclusive_sum(int64_t v, int64_t *total) {
  __shared__ int64_t warp_sums[SCAN_T / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    int64_t s = lane < SCAN_T / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < SCAN_T / 32) warp_sums[lane] = s;  // inclusive over warps
  }
  __syncthreads();
  const int64_t warp_base = w ? warp_sums[w - 1] : 0;
  if (total) *total = warp_sums[SCAN_T / 32 - 1];
  const int64_t excl = warp_base + x - v;
  __syncthreads();
  return excl;
}

__global__ void scan_tile_sums(const int64_t *in, int64_t n, int64_t *sums) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_V;
  int64_t s = 0;
#pragma unroll
  for (int q = 0; q < SCAN_V; q++)
    if (base + q < n) s += in[base + q];
  int64_t total;
  block_exclusive_sum(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_tiles(const int64_t *in, int64_t *out, int64_t n, const int64_t *tile_off,
                           int64_t *total_dev) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_V;
  int64_t v[SCAN_V], s = 0;
#pragma unroll
  for (int q = 0; q < SCAN_V; q++) {
    v[q] = base + q < n ? in[base + q] : 0;
    s += v[q];
  }
  int64_t total;
  int64_t run = block_exclusive_sum(s, &total) + (tile_off ? tile_off[blockIdx.x] : 0);
#pragma unroll
  for (int q = 0; q < SCAN_V; q++) {
    if (base + q < n) out[base + q] = run;
    run += v[q];
  }
  if (total_dev && blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_T - 1) *total_dev = run;
}

tq_status scan_exclusive(const int64_t *in, int64_t *out, int64_t n, int64_t *total_dev,
                         cudaStream_t s) {
  if (n <= 0) {
    if (total_dev) TQ_CUDA(cudaMemsetAsync(total_dev, 0, 8, s));
    return TQ_OK;
  }
  const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 1) {
    count_launch(), scan_tiles<<<1, SCAN_T, 0, s>>>(in, out, n, nullptr, total_dev);
    TQ_CUDA(cudaGetLastError());
    return TQ_OK;
  }
  DevArray<int64_t> sums, offs;
  TQ_CHECK(sums.alloc(tiles, s));
  TQ_CHECK(offs.alloc(tiles, s));
  count_launch(), scan_tile_sums<<<(unsigned)tiles, SCAN_T, 0, s>>>(in, n, sums.p);
  TQ_CUDA(cudaGetLastError());
  TQ_CHECK(scan_exclusive(sums.p, offs.p, tiles, nullptr, s));
  count_launch(), scan_tiles<<<(unsigned)tiles, SCAN_T, 0, s>>>(in, out, n, offs.p, total_dev);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

// ---------------------------------------------------------------- radix sort
// Stable LSD radix sort, 8-bit digits.  Tile = 256 threads x 16 rounds; within
// a tile elements are ranked in index order (round-major, then warp, then lane),
// which keeps equal keys in input order.
constexpr int RS_T = 256, RS_ROUNDS = 16, RS_TILE = RS_T * RS_ROUNDS;

__global__ void radix_hist(const int64_t *keys, int64_t n, int shift, int64_t *hist,
                           int64_t n_tiles) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; r++) {
    const int64_t i = base + r * RS_T + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255], 1);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * n_tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void radix_scatter(const int64_t *keys, const int64_t *vals, int64_t n, int shift,
                              const int64_t *offs, int64_t n_tiles, int64_t *okeys,
                              int64_t *ovals) {
  __shared__ int64_t run[256];
  __shared__ int cnt[RS_T / 32][256];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  run[t] = offs[(int64_t)t * n_tiles + blockIdx.x];
  for (int q = 0; q < RS_T / 32; q++) cnt[q][t] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < RS_ROUNDS; r++) {
    const int64_t i = base + r * RS_T + t;
    const bool valid = i < n;
    int64_t k = 0, v = 0;
    int d = 256;  // sentinel digit for lanes past the end
    if (valid) {
      k = keys[i];
      v = vals[i];
      d = (int)((k >> shift) & 255);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt);
    if (valid && rank == 0) cnt[w][d] = __popc(peers);
    __syncthreads();
    {  // thread t owns digit t: prefix over warps, advance the running offset
      int64_t x = run[t];
      for (int q = 0; q < RS_T / 32; q++) {
        const int c = cnt[q][t];
        cnt[q][t] = (int)(x - run[t]);
        x += c;
      }
      __syncthreads();
      if (valid) {
        const int64_t pos = run[d] + cnt[w][d] + rank;
        okeys[pos] = k;
        ovals[pos] = v;
      }
      __syncthreads();
      run[t] = x;
      for (int q = 0; q < RS_T / 32; q++) cnt[q][t] = 0;
      __syncthreads();
    }
  }
}

tq_status radix_sort_pairs(int64_t *keys, int64_t *vals, int64_t n, int key_bits,
                           cudaStream_t s) {
  if (n <= 1 || key_bits <= 0) return TQ_OK;
  const int64_t n_tiles = (n + RS_TILE - 1) / RS_TILE;
  DevArray<int64_t> k2, v2, hist, offs;
  TQ_CHECK(k2.alloc(n, s));
  TQ_CHECK(v2.alloc(n, s));
  TQ_CHECK(hist.alloc(256 * n_tiles, s));
  TQ_CHECK(offs.alloc(256 * n_tiles, s));
  int64_t *ka = keys, *va = vals, *kb = k2.p, *vb = v2.p;
  const int passes = (key_bits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    const int shift = 8 * p;
    count_launch(), radix_hist<<<(unsigned)n_tiles, RS_T, 0, s>>>(ka, n, shift, hist.p, n_tiles);
    TQ_CUDA(cudaGetLastError());
    TQ_CHECK(scan_exclusive(hist.p, offs.p, 256 * n_tiles, nullptr, s));
    count_launch(), radix_scatter<<<(unsigned)n_tiles, RS_T, 0, s>>>(ka, va, n, shift, offs.p, n_tiles, kb, vb);
    TQ_CUDA(cudaGetLastError());
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    TQ_CUDA(cudaMemcpyAsync(keys, ka, n * 8, cudaMemcpyDeviceToDevice, s));
    TQ_CUDA(cudaMemcpyAsync(vals, va, n * 8, cudaMemcpyDeviceToDevice, s));
  }
  return TQ_OK;
}

// ---------------------------------------------------------------- matching
// The interval test of block_in_range (src/tensor/block_sparse.cpp:42-60):
// B block j partners A block i iff, on every contracted leg,
// max(begin) <= min(end).  B's contracted intervals are gathered first into
// leg-major arrays so the per-lane loads are coalesced; each warp scans all B
// blocks for one A block and counts or emits matches with ballots, in
// ascending B order.

__global__ void gather_intervals(DevBS B, LegSpec legs, int64_t *lo, int64_t *hi) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= B.nb) return;
  for (int k = 0; k < legs.nc; k++) {
    lo[(int64_t)k * B.nb + j] = B.begin[j * B.rank + legs.bl[k]];
    hi[(int64_t)k * B.nb + j] = B.end[j * B.rank + legs.bl[k]];
  }
}

template <bool EMIT>
__global__ void match_kernel(DevBS A, int64_t nB, LegSpec legs, const int64_t *lo,
                             const int64_t *hi, int64_t *counts, const int64_t *row_off,
                             int32_t *pa, int32_t *pb) {
  const int lane = threadIdx.x & 31;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= A.nb) return;  // whole warp exits together
  int64_t alo[TQ_MAXR], ahi[TQ_MAXR];
#pragma unroll
  for (int k = 0; k < TQ_MAXR; k++)
    if (k < legs.nc) {
      alo[k] = A.begin[i * A.rank + legs.al[k]];
      ahi[k] = A.end[i * A.rank + legs.al[k]];
    }
  int64_t n = 0, out = EMIT ? row_off[i] : 0;
  const unsigned lt = (1u << lane) - 1u;
  for (int64_t base = 0; base < nB; base += 32) {
    const int64_t j = base + lane;
    bool ok = j < nB;
#pragma unroll
    for (int k = 0; k < TQ_MAXR; k++)
      if (k < legs.nc && ok) {
        const int64_t bl = lo[(int64_t)k * nB + j], bh = hi[(int64_t)k * nB + j];
        const int64_t mlo = alo[k] > bl ? alo[k] : bl;
        const int64_t mhi = ahi[k] < bh ? ahi[k] : bh;
        ok = mlo <= mhi;
      }
    const unsigned b = __ballot_sync(0xffffffffu, ok);
    if (EMIT && ok) {
      const int64_t p = out + __popc(b & lt);
      pa[p] = (int32_t)i;
      pb[p] = (int32_t)j;
    }
    out += __popc(b);
    n += __popc(b);
  }
  if (!EMIT && lane == 0) counts[i] = n;
}

struct IntervalCache {
  DevArray<int64_t> lo, hi;
};

static tq_status gather(const DevBS &B, const LegSpec &legs, IntervalCache &c, cudaStream_t s) {
  TQ_CHECK(c.lo.alloc((size_t)legs.nc * B.nb, s));
  TQ_CHECK(c.hi.alloc((size_t)legs.nc * B.nb, s));
  if (B.nb) {
    count_launch(), gather_intervals<<<(unsigned)((B.nb + 255) / 256), 256, 0, s>>>(B, legs, c.lo.p, c.hi.p);
    TQ_CUDA(cudaGetLastError());
  }
  return TQ_OK;
}

tq_status match_pairs(const DevBS &A, const DevBS &B, const LegSpec &legs, int64_t *counts,
                      cudaStream_t s) {
  if (A.nb == 0) return TQ_OK;
  IntervalCache c;
  TQ_CHECK(gather(B, legs, c, s));
  const int64_t threads = A.nb * 32;
  count_launch(), match_kernel<false><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
      A, B.nb, legs, c.lo.p, c.hi.p, counts, nullptr, nullptr, nullptr);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

tq_status emit_pairs(const DevBS &A, const DevBS &B, const LegSpec &legs, const int64_t *row_off,
                     int32_t *pa, int32_t *pb, cudaStream_t s) {
  if (A.nb == 0) return TQ_OK;
  IntervalCache c;
  TQ_CHECK(gather(B, legs, c, s));
  const int64_t threads = A.nb * 32;
  count_launch(), match_kernel<true><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
      A, B.nb, legs, c.lo.p, c.hi.p, nullptr, row_off, pa, pb);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

}  // namespace tq

extern "C" tq_status tq_nest_sum(const int64_t *counts, int64_t n, int64_t *offsets,
                                 int64_t *total, tq_stream stream) {
  if (n < 0) return tq::fail(TQ_ERR_INVALID, "negative length");
  if ((n > 0 && (!counts || !offsets)) || !total)
    return tq::fail(TQ_ERR_INVALID, "NULL argument");
  return tq::scan_exclusive(counts, offsets, n, total, (cudaStream_t)stream);
}

// ---------------------------------------------------------------- nest_sum without allocation
// Some callers cannot call cudaMalloc: code that owns all device memory through
// a fixed arena reserved at start-up, and latency-critical loops in which an
// allocation may block or synchronise the device.  tq_nest_sum_noalloc serves
// them: the same three-phase scan as tq_nest_sum, its tile sums and tile
// offsets kept in the file-scope array below instead of allocated scratch.
// Limit: TQ_NOALLOC_MAX_TILES tiles of SCAN_TILE counts, i.e. 4,194,304 counts.
// Every GPU that loads this library holds the 32 KB array until the process
// exits; every call shares it, so calls that overlap on the GPU race.  Each call
// writes every scratch entry it reads before reading it, so nothing has to be
// cleared between calls.
namespace tq {

constexpr int64_t TQ_NOALLOC_MAX_TILES = 2048;
constexpr int64_t TQ_NOALLOC_MAX_N = TQ_NOALLOC_MAX_TILES * SCAN_TILE;

static __device__ __align__(256) int64_t g_noalloc_scan[2 * TQ_NOALLOC_MAX_TILES];

// Device address of g_noalloc_scan, looked up once per device with that device
// current (in host code the symbol itself is only a host-side stand-in).
static std::mutex g_noalloc_mu;
static int64_t *g_noalloc_addr[128] = {nullptr};

static tq_status noalloc_scratch(int64_t **out) {
  int dev = 0;
  TQ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(TQ_ERR_UNSUPPORTED, "device ordinal above 127");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scan)");
    g_noalloc_addr[dev] = (int64_t *)p;
  }
  *out = g_noalloc_addr[dev];
  return TQ_OK;
}

}  // namespace tq

extern "C" tq_status tq_nest_sum_noalloc(const int64_t *counts, int64_t n, int64_t *offsets,
                                         int64_t *total, tq_stream stream) {
  using namespace tq;
  if (n < 0) return fail(TQ_ERR_INVALID, "negative length");
  if ((n > 0 && (!counts || !offsets)) || !total)
    return fail(TQ_ERR_INVALID, "NULL argument");
  if (n > TQ_NOALLOC_MAX_N)
    return fail(TQ_ERR_INVALID, "tq_nest_sum_noalloc takes at most 4194304 counts (got " +
                                    std::to_string(n) + "); use tq_nest_sum");
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    TQ_CUDA(cudaMemsetAsync(total, 0, 8, s));
    return TQ_OK;
  }
  const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 1) {
    count_launch(), scan_tiles<<<1, SCAN_T, 0, s>>>(counts, offsets, n, nullptr, total);
    TQ_CUDA(cudaGetLastError());
    return TQ_OK;
  }
  int64_t *scratch = nullptr;
  TQ_CHECK(noalloc_scratch(&scratch));
  int64_t *sums = scratch, *offs = scratch + TQ_NOALLOC_MAX_TILES;
  count_launch(), scan_tile_sums<<<(unsigned)tiles, SCAN_T, 0, s>>>(counts, n, sums);
  count_launch(), scan_tiles<<<1, SCAN_T, 0, s>>>(sums, offs, tiles, nullptr, nullptr);
  count_launch(), scan_tiles<<<(unsigned)tiles, SCAN_T, 0, s>>>(counts, offsets, n, offs, total);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}
