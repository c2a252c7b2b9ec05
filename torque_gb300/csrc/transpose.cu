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
// tiles.  Tiles are walked by a persistent grid sized by the kernel's
// occupancy; one load finds a tile's block.
//
// Two kernels.  4- and 8-byte elements take transpose_async_kernel: a CTA
// copies tile t+1 into the second of two shared stages with cp.async while it
// writes tile t out of the first, so HBM always has loads in flight; each
// block's description (sizes, strides, tiling, fast-divide constants) is
// computed once per call by describe_kernel instead of once per tile.  Half
// (no 2-byte cp.async) takes transpose_kernel, which stages its loads in
// registers (16-byte loads where a tile's input is one contiguous range).
// The output's device metadata and the first tile of each block are built on
// the device, so a call uploads nothing.
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
  const int64_t *out_strides; // output strides (n_blocks x rank, output leg order)
  int32_t inv[TQ_MAXR];       // output position of each input leg
  const int32_t *tile_block;  // [n_tiles] block of each tile
  int64_t nb;
  int32_t inv0;               // output position of input leg 0
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

// d0, dp: sizes of input leg 0 and of the leg that becomes output leg 0;
// rows: product of the other legs
__host__ __device__ inline PlanePlan plane_plan_of(uint32_t d0, uint32_t dp, uint64_t rows, int p0,
                                                   uint32_t cap, uint32_t pmax) {
  PlanePlan pp;
  pp.rows = (uint32_t)rows;
  if (p0 == 0) {
    pp.mode = 0;
    pp.P = d0;
    uint32_t ppc = cap / (d0 ? d0 : 1);
    ppc = ppc < 1 ? 1 : (ppc > pmax ? pmax : ppc);
    pp.ppc = ppc;
    pp.tiles = d0 > cap ? (int64_t)rows * ((d0 + cap - 1) / cap)
                        : (int64_t)((rows + ppc - 1) / ppc);
    return pp;
  }
  const uint64_t P = (uint64_t)(d0 + 1) * dp;  // leg-0 runs padded by one
  if (P <= (uint64_t)cap) {
    pp.mode = 1;
    pp.P = (uint32_t)P;
    uint32_t ppc = cap / pp.P;
    pp.ppc = ppc > pmax ? pmax : ppc;
    pp.tiles = (int64_t)((rows + pp.ppc - 1) / pp.ppc);
    return pp;
  }
  pp.mode = 2;
  pp.P = 0;
  pp.ppc = 1;
  pp.tiles = (int64_t)((d0 + TT - 1) / TT) * ((dp + TT - 1) / TT) * (int64_t)rows;
  return pp;
}

__host__ __device__ inline PlanePlan plane_plan(const uint32_t *d, int r, int p0,
                                               uint32_t cap = PLANE_MAX, uint32_t pmax = PLANES_MAX) {
  uint64_t rows = 1;
  for (int l = 1; l < r; l++)
    if (l != p0) rows *= d[l];
  return plane_plan_of(d[0], d[p0], rows, p0, cap, pmax);
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
__host__ __device__ inline uint32_t small_div_magic(uint32_t d) {
  return d > 1 ? 0xFFFFFFFFu / d + 1u : 0u;
}
struct SmallDiv {
  uint32_t d, m;
  __device__ __forceinline__ explicit SmallDiv(uint32_t dd) : d(dd), m(small_div_magic(dd)) {}
  __device__ __forceinline__ SmallDiv(uint32_t dd, uint32_t mm) : d(dd), m(mm) {}
  __device__ __forceinline__ uint32_t div(uint32_t x) const { return d > 1 ? __umulhi(x, m) : x; }
};

template <typename T>
__global__ void __launch_bounds__(256, 4) transpose_kernel(TransposeJob job, int64_t n_tiles) {
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
    // input of the tile = one contiguous range: dense column-major strides and
    // planes of legs (0) or (0, 1), so consecutive planes follow each other
    bool dense = true;
    {
      int64_t sacc = 1;
      for (int l = 0; l < r; l++) {
        dense = dense && st[l] == sacc;
        sacc *= d[l];
      }
    }
    const bool contig = dense && p0 <= 1;
    __syncthreads();
    const uint32_t d0 = d[0], dp = d[p0];
    const uint32_t PL = pp.mode == 0 ? d0 : d0 * dp;  // elements of one plane
    const uint32_t n = nrows * PL;                    // <= PLANE_MAX
    const SmallDiv by_pl(PL), by_d0(d0), by_dp(dp);
    constexpr int G = sizeof(T) == 8 ? 4 : 8;
    if (contig) {
      // element e of the tile is input element ib0 + row0 * PL + e, in plane e / PL
      const T *s0p = src + ib0 + (int64_t)row0 * PL;
      constexpr int V = 16 / (int)sizeof(T);
      uint32_t head = (uint32_t)(((16u - ((uint32_t)(uintptr_t)s0p & 15u)) & 15u) / sizeof(T));
      head = head > n ? n : head;
      const uint32_t nv = (n - head) / V, tail0 = head + nv * V;
      // the scalar head and tail (fewer than V elements each)
      uint32_t e1 = n;
      if ((uint32_t)tid < head) e1 = tid;
      else if ((uint32_t)tid - head < n - tail0) e1 = tail0 + tid - head;
      if (e1 < n) {
        const uint32_t pi = by_pl.div(e1), w = e1 - pi * PL;
        if (pp.mode == 0) {
          dst[base_out[pi] + w * o0] = s0p[e1];
        } else {
          const uint32_t j = by_d0.div(w), i = w - j * d0;
          buf[pi * pp.P + i + j * (d0 + 1)] = s0p[e1];
        }
      }
      const uint4 *vp = reinterpret_cast<const uint4 *>(s0p + head);
      for (uint32_t v0 = 0; v0 < nv; v0 += 4 * 256) {
        uint4 x[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const uint32_t v = v0 + k * 256 + tid;
          if (v < nv) x[k] = __ldcs(vp + v);
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const uint32_t v = v0 + k * 256 + tid;
          if (v < nv) {
            const T *xe = reinterpret_cast<const T *>(&x[k]);
            // decode the vector's first element once, then step
            const uint32_t e = head + v * V;
            uint32_t pi = by_pl.div(e), w = e - pi * PL;
            if (pp.mode == 0) {
#pragma unroll
              for (int q = 0; q < V; q++) {
                dst[base_out[pi] + w * o0] = xe[q];
                if (++w == PL) {
                  w = 0;
                  pi++;
                }
              }
            } else {
              uint32_t j = by_d0.div(w), i = w - j * d0;
#pragma unroll
              for (int q = 0; q < V; q++) {
                buf[pi * pp.P + i + j * (d0 + 1)] = xe[q];
                if (++i == d0) {
                  i = 0;
                  if (++j == dp) {
                    j = 0;
                    pi++;
                  }
                }
              }
            }
          }
        }
      }
      if (pp.mode == 0) continue;
    } else if (pp.mode == 0) {
      for (uint32_t e0 = 0; e0 < n; e0 += G * 256) {
        T x[G];
#pragma unroll
        for (int k = 0; k < G; k++) {
          const uint32_t e = e0 + k * 256 + tid;
          if (e < n) {
            const uint32_t pi = by_pl.div(e), i = e - pi * PL;
            x[k] = src[base_in[pi] + i * s0];
          }
        }
#pragma unroll
        for (int k = 0; k < G; k++) {
          const uint32_t e = e0 + k * 256 + tid;
          if (e < n) {
            const uint32_t pi = by_pl.div(e), i = e - pi * PL;
            dst[base_out[pi] + i * o0] = x[k];
          }
        }
      }
      continue;
    } else {
      for (uint32_t e0 = 0; e0 < n; e0 += G * 256) {
        T x[G];
#pragma unroll
        for (int k = 0; k < G; k++) {
          const uint32_t e = e0 + k * 256 + tid;
          if (e < n) {
            const uint32_t pi = by_pl.div(e), w = e - pi * PL, j = by_d0.div(w), i = w - j * d0;
            x[k] = src[base_in[pi] + i * s0 + j * sp];
          }
        }
#pragma unroll
        for (int k = 0; k < G; k++) {
          const uint32_t e = e0 + k * 256 + tid;
          if (e < n) {
            const uint32_t pi = by_pl.div(e), w = e - pi * PL, j = by_d0.div(w), i = w - j * d0;
            buf[pi * pp.P + i + j * (d0 + 1)] = x[k];
          }
        }
      }
    }
    __syncthreads();
    // planes out of the buffer along output leg 0 (input leg p0)
    for (uint32_t f = tid; f < n; f += 256) {
      const uint32_t pi = by_pl.div(f), w = f - pi * PL, i = by_dp.div(w), j = w - i * dp;
      __stcs(dst + base_out[pi] + j * op + i * o0, buf[pi * pp.P + i + j * (d0 + 1)]);
    }
  }
}


// ---------------------------------------------------------------------------
// Double-buffered form for 4- and 8-byte elements.  The register-staged kernel
// above leaves no load in flight while a tile is written out (load, barrier,
// store, barrier), so HBM idles half the time.  Here a CTA copies tile t+1
// into the second of two shared stages with cp.async (global -> shared, no
// register staging, completion tracked per commit group) while it writes tile
// t out of the first.  Runs that are contiguous in the input move as 16-byte
// copies into a stage shifted to the input's alignment; plane elements move
// as single-element copies into the padded plane layout (conflict-free on
// both sides).  Planes larger than a stage and runs longer than a stage take
// the unstaged paths (32 x 32 tiles, straight copies) in their turn.
constexpr int ACAP = 3072;    // elements per stage
constexpr int APLANES = 128;  // planes per tile
constexpr int AT = 128;       // threads per CTA (fewer threads amortise each tile's set-up over more elements)

// Everything a tile needs about its block, computed once per call by
// describe_kernel; a tile reads it with six 16-byte loads.
struct __align__(16) BlockDesc {
  int64_t ib0, ob0;  // data offsets of the block in the input and the output
  int64_t s0, sp;    // input strides of leg 0 and of leg p0
  int64_t o0;        // output stride of input leg 0 (output leg 0 has stride 1)
  int64_t tile0;     // first tile of the block
  uint32_t d0, dp, PL, P, ppc, rows;
  uint32_t m_pl, m_d0, m_dp;  // SmallDiv multipliers of PL, d0 and dp
  uint32_t flags;             // bits 0-1 mode, bit 2 contiguous input, bit 3 unstaged
  uint32_t pad[2];
};
constexpr uint32_t F_CONTIG = 4, F_DIRECT = 8;

// input and output offsets of plane `row` of block b (the legs other than 0
// and p0, in input order, lowest leg fastest); the leg loops are unrolled so
// the permutation is read from the kernel parameters at constant positions
__device__ __forceinline__ void plane_bases_of(const TransposeJob &job, int64_t b, uint32_t row,
                                               int64_t &ib, int64_t &ob) {
  const int r = job.rank, p0 = job.perm[0];
  const int64_t *bb = job.in.begin + b * r, *be = job.in.end + b * r, *st = job.in.strides + b * r;
  const int64_t *ost = job.out_strides + b * r;
#pragma unroll
  for (int l = 1; l < TQ_MAXR; l++) {
    if (l >= r || l == p0) continue;
    const uint32_t dl = (uint32_t)(be[l] - bb[l] + 1);
    const uint32_t c = row % dl;
    row /= dl;
    ib += c * st[l];
    ob += c * ost[job.inv[l]];
  }
}

// The output's metadata from the input's, on the device: boxes permuted,
// column-major strides, element counts (their exclusive scan gives the
// offsets) and the tiles of each block (their scan gives the first tiles).
__global__ void out_meta_kernel(TransposeJob job, int64_t *out_meta, int64_t *sizes, int64_t *tiles,
                                uint32_t cap, uint32_t pmax) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= job.nb) return;
  const int r = job.rank, p0 = job.perm[0];
  const int64_t nr = job.nb * r;
  const int64_t *bb = job.in.begin + b * r, *be = job.in.end + b * r;
  int64_t *ob = out_meta + b * r, *oe = out_meta + nr + b * r, *os = out_meta + 2 * nr + b * r;
  int64_t sacc = 1;
  uint64_t rows = 1;
#pragma unroll
  for (int q = 0; q < TQ_MAXR; q++) {
    if (q >= r) continue;
    const int l = job.perm[q];
    ob[q] = bb[l];
    oe[q] = be[l];
    os[q] = sacc;
    const int64_t dl = be[l] - bb[l] + 1;
    sacc *= dl;
    if (q > 0 && l != 0) rows *= (uint64_t)dl;
  }
  sizes[b] = sacc;
  const uint32_t d0 = (uint32_t)(be[0] - bb[0] + 1), dp = (uint32_t)(be[p0] - bb[p0] + 1);
  tiles[b] = plane_plan_of(d0, dp, rows, p0, cap, pmax).tiles;
}

__global__ void describe_kernel(TransposeJob job, BlockDesc *descs) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= job.nb) return;
  const int r = job.rank, p0 = job.perm[0];
  const int64_t *bb = job.in.begin + b * r, *be = job.in.end + b * r, *st = job.in.strides + b * r;
  uint64_t rows = 1;
  bool dense = true;
  int64_t sacc = 1;
  uint32_t d0 = 1, dp = 1;
#pragma unroll
  for (int l = 0; l < TQ_MAXR; l++) {
    if (l >= r) continue;
    const uint32_t dl = (uint32_t)(be[l] - bb[l] + 1);
    if (l == 0) d0 = dl;
    if (l == p0) dp = dl;
    if (l != 0 && l != p0) rows *= dl;
    dense = dense && st[l] == sacc;
    sacc *= dl;
  }
  const PlanePlan pp = plane_plan_of(d0, dp, rows, p0, ACAP, APLANES);
  const bool direct = pp.mode == 2 || (pp.mode == 0 && d0 > (uint32_t)ACAP);
  BlockDesc D;
  D.ib0 = job.in.offsets[b];
  D.ob0 = job.out_off[b];
  D.s0 = st[0];
  D.sp = st[p0];
  D.o0 = job.out_strides[b * r + job.inv0];
  D.tile0 = job.tile_start[b];
  D.d0 = d0;
  D.dp = dp;
  D.PL = pp.mode == 0 ? d0 : d0 * dp;
  D.P = pp.P;
  D.ppc = pp.ppc;
  D.rows = pp.rows;
  // the multipliers are exact for quotients of in-tile indices (< ACAP) by
  // divisors up to ACAP: only staged tiles use them
  D.m_pl = direct ? 0u : small_div_magic(D.PL);
  D.m_d0 = direct ? 0u : small_div_magic(d0);
  D.m_dp = direct ? 0u : small_div_magic(dp);
  // consecutive planes of legs (0) or (0, 1) follow each other in the input
  D.flags = (uint32_t)pp.mode | (dense && p0 <= 1 ? F_CONTIG : 0u) | (direct ? F_DIRECT : 0u);
  D.pad[0] = D.pad[1] = 0;
  descs[b] = D;
}

struct StageInfo {
  uint32_t direct, mode, P, PL, d0, dp, n, sh, m_pl, m_dp;
  int64_t o0;
};

template <int BYTES>
__device__ __forceinline__ void cp_async(uint32_t dst, const void *src) {
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
  else if constexpr (BYTES == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

template <typename T>
__global__ void __launch_bounds__(AT, 4)
    transpose_async_kernel(TransposeJob job, const BlockDesc *__restrict__ descs, int64_t n_tiles) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cp.async moves 4, 8 or 16 bytes");
  constexpr int V = 16 / (int)sizeof(T);
  constexpr int STAGE = ACAP + V;  // room for the alignment shift, 16-byte multiple
  __shared__ __align__(16) T buf[2][STAGE];
  __shared__ int64_t bout[2][APLANES];
  __shared__ int64_t bin[APLANES];  // read only while a tile's copies are issued
  __shared__ StageInfo info[2];
  const T *__restrict__ src = (const T *)job.in.data;
  T *__restrict__ dst = (T *)job.out;
  const uint32_t tid = threadIdx.x;

  // plane output bases owed to the stage last prefetched: a contiguous tile
  // needs them only when it is written out, so they are computed after the
  // current tile's stores, off the path to the barrier
  int64_t owed_b = -1, owed_ob0 = 0;
  uint32_t owed_row0 = 0, owed_nrows = 0;
  auto pay_bases = [&](int s) {
    if (owed_b >= 0 && tid < owed_nrows) {
      int64_t ib = 0, ob = owed_ob0;
      plane_bases_of(job, owed_b, owed_row0 + tid, ib, ob);
      bout[s][tid] = ob;
    }
    owed_b = -1;
  };

  // start the copies of tile t into stage s (one commit group per call)
  auto prefetch = [&](int64_t t, int s) {
    const int64_t b = job.tile_block[t];
    const BlockDesc D = descs[b];
    if (!(D.flags & F_DIRECT)) {
      const bool contig = D.flags & F_CONTIG;
      const uint32_t mode = D.flags & 3u;
      const uint32_t row0 = (uint32_t)(t - D.tile0) * D.ppc;
      const uint32_t nrows = D.rows - row0 < D.ppc ? D.rows - row0 : D.ppc;
      const uint32_t PL = D.PL, d0 = D.d0, n = nrows * PL;  // n <= ACAP
      const T *s0p = src + D.ib0 + (int64_t)row0 * PL;
      const uint32_t sh = contig && mode == 0 ? (uint32_t)(((uintptr_t)s0p & 15u) / sizeof(T)) : 0u;
      if (contig) {
        owed_b = b;
        owed_ob0 = D.ob0;
        owed_row0 = row0;
        owed_nrows = nrows;
      } else if (tid < nrows) {
        int64_t ib = D.ib0, ob = D.ob0;
        plane_bases_of(job, b, row0 + tid, ib, ob);
        bin[tid] = ib;
        bout[s][tid] = ob;
      }
      if (tid == 0) {
        StageInfo I;
        I.direct = 0;
        I.mode = mode;
        I.P = D.P;
        I.PL = PL;
        I.d0 = d0;
        I.dp = D.dp;
        I.n = n;
        I.sh = sh;
        I.m_pl = D.m_pl;
        I.m_dp = D.m_dp;
        I.o0 = D.o0;
        info[s] = I;
      }
      if (!contig) __syncthreads();  // the plane bases address the copies
      const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(&buf[s][0]);
      const SmallDiv by_pl(PL, D.m_pl), by_d0(d0, D.m_d0);
      if (mode == 0 && contig) {
        // one contiguous run of n elements into buf[s][sh ..]: 16-byte copies
        // between the scalar head and tail
        const uint32_t h0 = (uint32_t)((V - sh) % V), h = h0 < n ? h0 : n;
        const uint32_t nv = (n - h) / V, tail0 = h + nv * V;
        if (tid < h) cp_async<sizeof(T)>(sbase + (sh + tid) * sizeof(T), s0p + tid);
        else if (tid - h < n - tail0)
          cp_async<sizeof(T)>(sbase + (sh + tail0 + tid - h) * sizeof(T), s0p + tail0 + tid - h);
        for (uint32_t c = tid; c < nv; c += AT)
          cp_async<16>(sbase + (sh + h + c * V) * sizeof(T), s0p + h + c * V);
      } else if (mode == 0) {
        for (uint32_t e = tid; e < n; e += AT) {
          const uint32_t pi = by_pl.div(e), i = e - pi * PL;
          cp_async<sizeof(T)>(sbase + e * sizeof(T), src + bin[pi] + i * D.s0);
        }
      } else if (contig) {
        // plane pi sits at buf[s][pi * P + i + j * (d0 + 1)]
        for (uint32_t e = tid; e < n; e += AT) {
          const uint32_t pi = by_pl.div(e), w = e - pi * PL, j = by_d0.div(w), i = w - j * d0;
          cp_async<sizeof(T)>(sbase + (pi * D.P + i + j * (d0 + 1)) * sizeof(T), s0p + e);
        }
      } else {
        for (uint32_t e = tid; e < n; e += AT) {
          const uint32_t pi = by_pl.div(e), w = e - pi * PL, j = by_d0.div(w), i = w - j * d0;
          cp_async<sizeof(T)>(sbase + (pi * D.P + i + j * (d0 + 1)) * sizeof(T),
                              src + bin[pi] + i * D.s0 + j * D.sp);
        }
      }
    } else if (tid == 0) {
      info[s].direct = 1;
    }
    cp_async_commit();
  };

  int64_t t = blockIdx.x;
  if (t >= n_tiles) return;
  int k = 0;
  prefetch(t, 0);
  pay_bases(0);
  for (; t < n_tiles; t += gridDim.x) {
    const int64_t tn = t + gridDim.x;
    // stage k^1 was last read by the previous tile's stores, which ended at
    // that iteration's closing barrier
    if (tn < n_tiles) prefetch(tn, k ^ 1);
    else cp_async_commit();
    cp_async_wait1();  // this thread's copies of tile t have landed
    __syncthreads();   // and every thread's
    const StageInfo I = info[k];
    if (I.direct) {
      const int64_t b = job.tile_block[t];
      const BlockDesc D = descs[b];
      const uint32_t local = (uint32_t)(t - D.tile0), d0 = D.d0, dp = D.dp;
      if ((D.flags & 3u) == 2u) {
        // one 32 x 32 tile of a large plane, through stage k
        const uint32_t n0 = (d0 + TT - 1) / TT, np = (dp + TT - 1) / TT;
        const uint32_t i0 = (local % n0) * TT, j0 = ((local / n0) % np) * TT;
        int64_t ib = D.ib0, ob = D.ob0;
        plane_bases_of(job, b, local / n0 / np, ib, ob);
        T(*tile)[TT + 1] = reinterpret_cast<T(*)[TT + 1]>(&buf[k][0]);
        const uint32_t tx = tid & 31, ty = tid >> 5;
        for (uint32_t q = ty; q < TT; q += AT / 32) {
          const uint32_t ii = i0 + tx, jj = j0 + q;
          if (ii < d0 && jj < dp) tile[q][tx] = src[ib + ii * D.s0 + jj * D.sp];
        }
        __syncthreads();
        for (uint32_t q = ty; q < TT; q += AT / 32) {
          const uint32_t jj = j0 + tx, ii = i0 + q;
          if (ii < d0 && jj < dp) dst[ob + jj + ii * D.o0] = tile[tx][q];
        }
      } else {
        // one ACAP-long piece of a long run
        const uint32_t npc = (d0 + ACAP - 1) / ACAP;
        const uint32_t i0 = (local % npc) * ACAP;
        int64_t ib = D.ib0, ob = D.ob0;
        plane_bases_of(job, b, local / npc, ib, ob);
        for (uint32_t i = i0 + tid; i < d0 && i < i0 + ACAP; i += AT)
          dst[ob + i * D.o0] = src[ib + i * D.s0];
      }
    } else if (I.mode == 0) {
      const SmallDiv by_pl(I.PL, I.m_pl);
      for (uint32_t f = tid; f < I.n; f += AT) {
        const uint32_t pi = by_pl.div(f), i = f - pi * I.PL;
        __stcs(dst + bout[k][pi] + i * I.o0, buf[k][I.sh + f]);
      }
    } else {
      // planes out along output leg 0 (input leg p0)
      const SmallDiv by_pl(I.PL, I.m_pl), by_dp(I.dp, I.m_dp);
      for (uint32_t f = tid; f < I.n; f += AT) {
        const uint32_t pi = by_pl.div(f), w = f - pi * I.PL, i = by_dp.div(w), j = w - i * I.dp;
        __stcs(dst + bout[k][pi] + j + i * I.o0, buf[k][pi * I.P + i + j * (I.d0 + 1)]);
      }
    }
    pay_bases(k ^ 1);  // bases of the tile now in flight
    __syncthreads();   // stage k is free again; the owed bases are visible
    k ^= 1;
  }
}

// The persistent grid is exactly the CTAs resident at once (a larger fixed
// grid would run its surplus CTAs as a second, mostly idle wave).
template <typename Kernel, typename... Args>
static tq_status launch_transpose(Kernel kernel, int threads, int64_t n_tiles, int sms,
                                  cudaStream_t s, Args... args) {
  int per_sm = 0;  // resident CTAs per SM
  TQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0));
  const unsigned grid = (unsigned)std::min<int64_t>(n_tiles, (int64_t)std::max(per_sm, 1) * sms);
  count_launch(), kernel<<<grid, threads, 0, s>>>(args..., n_tiles);
  return TQ_OK;
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
  if (t->nb) {
    // tiles per block from the host metadata (no device round trip)
    const int32_t p0 = (int32_t)perm[0];
    // 4- and 8-byte elements take the double-buffered kernel, half the
    // register-staged one (cp.async has no 2-byte copy); their tilings differ
    const bool staged = t->dtype != TQ_F16;
    const uint32_t cap = staged ? ACAP : PLANE_MAX, pmax = staged ? APLANES : PLANES_MAX;
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
      n_tiles += plane_plan(d, r, p0, cap, pmax).tiles;
    }
    if (n_tiles > 0x7fffffffLL) return fail(TQ_ERR_UNSUPPORTED, "more than 2^31 transpose tiles");
    if (t->nb > 0x7fffffffLL) return fail(TQ_ERR_UNSUPPORTED, "more than 2^31 blocks");
    DevArray<int64_t> tile_start, sizes, tiles;
    DevArray<int32_t> tile_block;
    DevArray<BlockDesc> descs;
    TQ_CHECK(tile_start.alloc(t->nb, s));
    TQ_CHECK(sizes.alloc(t->nb, s));
    TQ_CHECK(tiles.alloc(t->nb, s));
    TQ_CHECK(tile_block.alloc(std::max<int64_t>(n_tiles, 1), s));
    TQ_CHECK(o->d_meta.alloc(3 * t->nb * r + t->nb, s));
    TransposeJob job{};
    job.in = t->view();
    job.rank = r;
    for (int32_t l = 0; l < r; l++) job.perm[l] = (int32_t)perm[l];
    job.out_off = o->d_meta.p + 3 * o->nb * r;
    job.tile_start = tile_start.p;
    job.tile_block = tile_block.p;
    job.out_strides = o->d_meta.p + 2 * o->nb * r;
    for (int32_t l = 0; l < r; l++) job.inv[perm[l]] = l;
    job.inv0 = job.inv[0];
    job.nb = t->nb;
    job.out = o->data;
    // the output's device metadata and the first tile of each block are
    // built on the device (no host upload); the host copies above agree
    const unsigned mb = (unsigned)((t->nb + 255) / 256);
    count_launch(), out_meta_kernel<<<mb, 256, 0, s>>>(job, o->d_meta.p, sizes.p, tiles.p, cap, pmax);
    TQ_CHECK(scan_exclusive(sizes.p, o->d_meta.p + 3 * t->nb * r, t->nb, nullptr, s));
    TQ_CHECK(scan_exclusive(tiles.p, tile_start.p, t->nb, nullptr, s));
    o->dev_valid = true;
    if (n_tiles) {
      count_launch(), tile_block_kernel<<<(unsigned)t->nb, 256, 0, s>>>(tile_start.p, t->nb, n_tiles,
                                                                         tile_block.p);
      int dev = 0, sms = 0;
      TQ_CUDA(cudaGetDevice(&dev));
      TQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      // a transpose moves bits: the element size picks the kernel
      NvtxRange range("tq_transpose");
      if (staged) {
        TQ_CHECK(descs.alloc(t->nb, s));
        count_launch(), describe_kernel<<<(unsigned)((t->nb + 255) / 256), 256, 0, s>>>(job, descs.p);
      }
      if (t->dtype == TQ_F64)
        TQ_CHECK(launch_transpose(transpose_async_kernel<unsigned long long>, AT, n_tiles, sms, s,
                                  job, (const BlockDesc *)descs.p));
      else if (t->dtype == TQ_F32)
        TQ_CHECK(launch_transpose(transpose_async_kernel<unsigned>, AT, n_tiles, sms, s, job,
                                  (const BlockDesc *)descs.p));
      else
        TQ_CHECK(launch_transpose(transpose_kernel<unsigned short>, 256, n_tiles, sms, s, job));
      TQ_CUDA(cudaGetLastError());
    }
  }
  *out = guard.release();
  return TQ_OK;
}
