// Tensor-core forms of the grouped block GEMM: FP64-level ("Ozaki") and
// FP32-level (three-way bf16 split) products on tcgen05, fed by the TMA engine.
//
// Method (error-free splitting, Ozaki-Ogita-Oishi-Rump; integer-slice GEMM
// recombination as in Ootomo-Ozaki-Yokota 2024, with the slices carried in
// bf16 as in the FP16-tensor-core variant of Mukunoki-Ozaki-Ogita-Imamura 2020):
//   * every output row r has an exponent e_r (max over the whole fused row of
//     A: all A blocks sharing the output's free box) and every output column c
//     an exponent f_c (same for B), with |x| * 2^-e < 1/2;
//   * x * 2^(8s-e) is rounded to an integer F and split into s signed base-256
//     digits d_0..d_{s-1} in [-128, 128]; slice t is stored as the bf16 value
//     d_t * 2^(-8t) (exact: at most 8 significant bits);
//   * the slice products A_t B_u^T with t+u <= s-1 run on the tensor cores with
//     fp32 accumulation in TMEM, in five accumulators by g = t+u: D0..D3
//     (g = 0..3) hold multiples of 2^(-8g) below (g+1) K 2^14 2^(-8g), whole
//     numbers of 24 bits or fewer for K <= 240, so the tensor core sums them
//     exactly; D4 (g >= 4, at most 2^-32 of D0) is rounded.  Every 240 columns
//     of the fused K (all pairs of the output block, in order) the five are
//     folded into an int64 running sum S = sum_a round(2^24 D_a) held in the
//     epilogue's registers (exact but for D4's rounding; below 2^60 for a fused
//     K up to 2^20).  A single fp32 accumulator for the lower groups is not
//     enough: the tensor core's fp32 accumulation truncates, which loses about
//     K ulps of the group it holds.
//   * C = S * 2^(e_r + f_c - 40), converted to FP64 with integer operations.
// No FP64 arithmetic runs in the GEMM: GB300 issues about 2 FP64 FMAs per SM
// per clock against ~4000 bf16 FMAs, so FP64 work stays in the row-exponent
// pass (one ilogb per row) only.
//
// Layout of the sliced operands in global memory (built by oz_slice_kernel):
// for every operand block, row tiles of RT rows (128 for A, 96 for B); in a
// row tile, k-steps of 16 columns; in a k-step, s slices of G = ceil(rows/8)
// row groups; in a row group two 8x8 bf16 core matrices (k 0-7, 8-15) of 128
// contiguous bytes.  That is exactly the shared-memory image tcgen05 reads
// (K-major, no swizzle, LBO = 128 B along K, SBO = 256 B along M/N), so one
// bulk copy per operand per k-step fills a pipeline stage.
#include <cuda_bf16.h>

#include "gemm.cuh"
#include "ozaki.cuh"
#include "sm100_ptx.cuh"

namespace tq {

constexpr int OZ_THREADS = 320;  // warp 0: loads, warp 1: MMA, warps 2-9: epilogue
constexpr uint32_t OZ_TMEM_COLS = 512;
// TMEM columns: accumulator D_a (a = 0..4) at [a*OZ_N, (a+1)*OZ_N), 480 of 512
constexpr int OZ_NACC = 5;
static_assert(OZ_NACC * OZ_N <= (int)OZ_TMEM_COLS, "accumulators exceed TMEM");
constexpr int OZ_SMEM_BYTES = 200 * 1024;

__device__ __forceinline__ int64_t oz_find(const int64_t *start, int64_t n, int64_t t) {
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (start[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int64_t free_rows(const DevBS &T, int64_t b, int32_t nf,
                                             const int32_t *fl) {
  int64_t m = 1;
  for (int q = 0; q < nf; q++) m *= T.end[b * T.rank + fl[q]] - T.begin[b * T.rank + fl[q]] + 1;
  return m;
}

// ---------------------------------------------------------------- exponents
__global__ void oz_exp_init_kernel(int32_t *e, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) e[i] = OZ_EXP_ZERO;
}

// One thread per (block, row): max |x| over the row's contracted columns.
__global__ void oz_rowexp_kernel(OzSide S, int64_t total_rows, int32_t *exps) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_rows) return;
  const int64_t b = oz_find(S.row_start, S.T.nb, g);
  const int64_t r = g - S.row_start[b];
  Operand op;
  int64_t cb[TQ_MAXR], ce[TQ_MAXR];
  for (int k = 0; k < S.ncon; k++) {
    cb[k] = S.T.begin[b * S.T.rank + S.con[k]];
    ce[k] = S.T.end[b * S.T.rank + S.con[k]];
  }
  build_operand(S.T, b, S.nfree, S.free_legs, S.ncon, S.con, cb, ce, op);
  const double *d = (const double *)S.T.data;
  const int64_t ra = op.base + mixed_addr(r, op.nr, op.rdim, op.rst);
  unsigned long long mx = 0;
  for (int64_t k = 0; k < op.cols; k++) {
    const unsigned long long bits =
        (unsigned long long)__double_as_longlong(d[ra + mixed_addr(k, op.nc, op.cdim, op.cst)]) &
        0x7fffffffffffffffull;
    mx = bits > mx ? bits : mx;
  }
  if (mx == 0) return;
  const int e = ilogb(__longlong_as_double((long long)mx)) + 2;
  atomicMax(&exps[S.row_off[S.key[b]] + r], e);
}

// x * 2^shift rounded to the nearest integer (ties to even), integer ops only.
__device__ __forceinline__ long long oz_fixed(double x, int shift) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int ex = (int)((b >> 52) & 0x7ff);
  unsigned long long man = b & 0xfffffffffffffull;
  if (ex == 0) {
    if (man == 0) return 0;
    ex = 1;
  } else {
    man |= 1ull << 52;
  }
  const int sh = ex - 1075 + shift;
  unsigned long long q;
  if (sh >= 0) {
    q = man << sh;  // |x 2^shift| < 2^(8s-1) <= 2^55 by the choice of exponent
  } else if (sh < -54) {
    q = 0;
  } else {
    const int rs = -sh;
    q = man >> rs;
    const unsigned long long rem = man & ((1ull << rs) - 1), half = 1ull << (rs - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
  }
  return (b >> 63) ? -(long long)q : (long long)q;
}

// One CTA per (block, row tile): slices of all k-steps of the tile.
__global__ void __launch_bounds__(256) oz_slice_kernel(OzSide S, int32_t s, int32_t rt_rows,
                                                       const int32_t *exps, uint8_t *out) {
  const int64_t tile = blockIdx.x;
  const int64_t b = oz_find(S.tile_start, S.T.nb, tile);
  const int64_t rt = tile - S.tile_start[b];
  Operand op;
  int64_t cb[TQ_MAXR], ce[TQ_MAXR];
  for (int k = 0; k < S.ncon; k++) {
    cb[k] = S.T.begin[b * S.T.rank + S.con[k]];
    ce[k] = S.T.end[b * S.T.rank + S.con[k]];
  }
  build_operand(S.T, b, S.nfree, S.free_legs, S.ncon, S.con, cb, ce, op);
  const int64_t rows = op.rows - rt * rt_rows < rt_rows ? op.rows - rt * rt_rows : rt_rows;
  const int G = (int)((rows + 7) / 8);
  const int64_t nk = (op.cols + 15) / 16;
  uint8_t *base = out + 256 * S.unit_off[b] + nk * (int64_t)s * 256 * (rt_rows / 8) * rt;
  const double *d = (const double *)S.T.data;
  const int r = threadIdx.x >> 1, c = threadIdx.x & 1;
  if (r >= G * 8) return;
  const int64_t grow = rt * rt_rows + r;
  const bool row_ok = r < rows;
  const int e = row_ok ? exps[S.row_off[S.key[b]] + grow] : OZ_EXP_ZERO;
  const int shift = 8 * s - e;
  const int64_t ra = row_ok ? op.base + mixed_addr(grow, op.nr, op.rdim, op.rst) : 0;
  for (int64_t q = 0; q < nk; q++) {
    uint8_t *chunk = base + q * (int64_t)s * G * 256;
    uint32_t packed[OZ_MAXS][4];
#pragma unroll
    for (int t = 0; t < OZ_MAXS; t++)
#pragma unroll
      for (int w = 0; w < 4; w++) packed[t][w] = 0;
#pragma unroll
    for (int x = 0; x < 8; x++) {
      const int64_t k = q * 16 + c * 8 + x;
      long long F = 0;
      if (row_ok && k < op.cols) F = oz_fixed(d[ra + mixed_addr(k, op.nc, op.cdim, op.cst)], shift);
      int dig[OZ_MAXS];
#pragma unroll
      for (int t = OZ_MAXS - 1; t >= 1; t--) {
        if (t < s) {
          const int dd = (int)(((F + 128) & 255) - 128);
          dig[t] = dd;
          F = (F - dd) >> 8;
        } else {
          dig[t] = 0;
        }
      }
      dig[0] = (int)F;
#pragma unroll
      for (int t = 0; t < OZ_MAXS; t++) {
        // d_t * 2^(-8t), exact in bf16
        const float v = (float)dig[t] * __int_as_float((127 - 8 * t) << 23);
        const uint32_t h = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v));
        packed[t][x >> 1] |= h << (16 * (x & 1));
      }
    }
#pragma unroll
    for (int t = 0; t < OZ_MAXS; t++) {
      if (t >= s) break;
      uint4 v = make_uint4(packed[t][0], packed[t][1], packed[t][2], packed[t][3]);
      *(uint4 *)(chunk + ((t * G + r / 8) * 2 + c) * 128 + (r % 8) * 16) = v;
    }
  }
}

// ---------------------------------------------------------------- conversion
// T * 2^e as a correctly rounded double, integer operations only (the rare
// out-of-range exponents take the FP64 path).
__device__ __forceinline__ double oz_i64_ldexp(long long T, int e) {
  if (T == 0) return 0.0;
  const unsigned long long sign = T < 0 ? (1ull << 63) : 0ull;
  unsigned long long a = T < 0 ? (unsigned long long)(-T) : (unsigned long long)T;
  int msb = 63 - __clzll((long long)a);
  unsigned long long mant;
  if (msb <= 52) {
    mant = a << (52 - msb);
  } else {
    const int sh = msb - 52;
    unsigned long long q = a >> sh;
    const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    if (q >> 53) {
      q >>= 1;
      msb++;
    }
    mant = q;
  }
  const int be = msb + e + 1023;
  if (be <= 0 || be >= 2047) return ldexp((double)T, e);
  return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) |
                                          (mant & 0xfffffffffffffull)));
}

// ---------------------------------------------------------------- the GEMM
// All slice products of one k-step, fully unrolled: product (t, u) goes to
// accumulator min(t+u, OZ_NACC-1).  Descriptors advance by whole row groups
// (the start-address field counts 16-byte units).  On the first k-step of a
// flush chunk the first product into each accumulator overwrites it.
template <int S>
__device__ __forceinline__ void oz_issue(uint32_t tmem, uint64_t da0, uint64_t db0,
                                         uint32_t a_step, uint32_t b_step, uint32_t idesc,
                                         bool chunk_start) {
#pragma unroll
  for (int t = 0; t < S; t++) {
#pragma unroll
    for (int u = 0; u < S - t; u++) {
      const int acc = t + u < OZ_NACC - 1 ? t + u : OZ_NACC - 1;
      // first (t, u) in this order that lands in accumulator acc
      const bool first = acc < OZ_NACC - 1 ? t == 0 : (t == 0 && u == OZ_NACC - 1);
      mma_bf16(tmem + acc * OZ_N, da0 + (uint64_t)(t * a_step), db0 + (uint64_t)(u * b_step),
               idesc, (chunk_start && first) ? 0u : 1u);
    }
  }
}

__device__ __forceinline__ void oz_issue_s(int s, uint32_t tmem, uint64_t da0, uint64_t db0,
                                           uint32_t a_step, uint32_t b_step, uint32_t idesc,
                                           bool chunk_start) {
  switch (s) {
    case 1: oz_issue<1>(tmem, da0, db0, a_step, b_step, idesc, chunk_start); break;
    case 2: oz_issue<2>(tmem, da0, db0, a_step, b_step, idesc, chunk_start); break;
    case 3: oz_issue<3>(tmem, da0, db0, a_step, b_step, idesc, chunk_start); break;
    case 4: oz_issue<4>(tmem, da0, db0, a_step, b_step, idesc, chunk_start); break;
    case 5: oz_issue<5>(tmem, da0, db0, a_step, b_step, idesc, chunk_start); break;
    case 6: oz_issue<6>(tmem, da0, db0, a_step, b_step, idesc, chunk_start); break;
    default: oz_issue<7>(tmem, da0, db0, a_step, b_step, idesc, chunk_start); break;
  }
}

// Exact fp32 -> int32 for values whose scaled magnitude is below 2^22 (one FMA
// against 1.5 * 2^23, whose ulp is 1, then an integer subtract; rounds to
// nearest even like rint); larger values take the conversion unit.
__device__ __forceinline__ int oz_to_int(float x, float scale) {
  const float y = x * scale;
  if (fabsf(y) < 4194304.0f) return __float_as_int(y + 12582912.0f) - 0x4B400000;
  return __float2int_rn(y);
}

struct OzTile {
  int64_t o, mt, nt, m, n, i0, j0, seg0, seg1, ksum;
  int32_t ga, gb, nmma;
};

__device__ __forceinline__ void oz_decode(const OzJob &J, int64_t t, OzTile &T) {
  T.o = oz_find(J.tile_start, J.g.n_out, t);
  T.seg0 = J.g.seg[T.o];
  T.seg1 = J.g.seg[T.o + 1];
  const int64_t p0 = J.g.perm ? J.g.perm[T.seg0] : T.seg0;
  T.i0 = J.g.pa[p0];
  T.j0 = J.g.pb[p0];
  T.m = free_rows(J.g.A, T.i0, J.g.L.nfa, J.g.L.fa);
  T.n = free_rows(J.g.B, T.j0, J.g.L.nfb, J.g.L.fb);
  const int64_t tiles_m = (T.m + OZ_M - 1) / OZ_M;
  const int64_t local = t - J.tile_start[T.o];
  T.mt = local % tiles_m;
  T.nt = local / tiles_m;
  const int64_t ra = min((int64_t)OZ_M, T.m - T.mt * OZ_M);
  const int64_t rb = min((int64_t)OZ_N, T.n - T.nt * OZ_N);
  T.ga = (int32_t)((ra + 7) / 8);
  T.gb = (int32_t)((rb + 7) / 8);
  T.nmma = (int32_t)(16 * ((rb + 15) / 16));
  T.ksum = J.ksum[T.o];
}

__global__ void __launch_bounds__(OZ_THREADS, 1) oz_gemm_kernel(OzJob J) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full_bar[OZ_MAX_STAGES], empty_bar[OZ_MAX_STAGES];
  __shared__ __align__(8) uint64_t acc_full, acc_empty, done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = J.s, NS = J.nstages;
  const uint32_t a_bytes_max = (uint32_t)s * (OZ_M / 8) * 256;
  const uint32_t stage_bytes = (uint32_t)s * ((OZ_M + OZ_N) / 8) * 256;

  if (threadIdx.x == 0) {
    for (int q = 0; q < NS; q++) {
      mbar_init(&full_bar[q], 1);
      mbar_init(&empty_bar[q], 1);
    }
    mbar_init(&acc_full, 1);
    mbar_init(&acc_empty, 8);
    mbar_init(&done_bar, 1);
    abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&tmem_base, OZ_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == 0) {
    // ---------------- producer: one bulk copy per operand per k-step
    if (lane == 0) {
      uint32_t it = 0;
      for (int64_t t = blockIdx.x; t < J.n_tiles && !abort_flag; t += gridDim.x) {
        OzTile T;
        oz_decode(J, t, T);
        const uint32_t ba = (uint32_t)s * T.ga * 256, bb = (uint32_t)s * T.gb * 256;
        for (int64_t sidx = T.seg0; sidx < T.seg1 && !abort_flag; sidx++) {
          const int64_t p = J.g.perm ? J.g.perm[sidx] : sidx;
          const int64_t i = J.g.pa[p], j = J.g.pb[p];
          const int64_t nk = J.nk_pair[p];
          const uint8_t *ga = J.sliceA + 256 * J.unitA[i] + nk * s * 256 * (OZ_M / 8) * T.mt;
          const uint8_t *gb = J.sliceB + 256 * J.unitB[j] + nk * s * 256 * (OZ_N / 8) * T.nt;
          for (int64_t q = 0; q < nk; q++, it++) {
            const uint32_t st = it % NS, use = it / NS;
            if (use > 0 && !mbar_wait(&empty_bar[st], (use - 1) & 1)) {
              atomicOr(J.err, 1);
              abort_flag = 1;
              break;
            }
            uint8_t *sa = smem + st * stage_bytes;
            mbar_arrive_expect_tx(&full_bar[st], ba + bb);
            bulk_g2s(sa, ga + q * ba, ba, &full_bar[st]);
            bulk_g2s(sa + a_bytes_max, gb + q * bb, bb, &full_bar[st]);
          }
        }
      }
      // drain: every copy issued must land before the CTA may exit
      const uint32_t first = it > (uint32_t)NS ? it - NS : 0;
      for (uint32_t q = first; q < it; q++) {
        if (!mbar_wait(&full_bar[q % NS], (q / NS) & 1)) atomicOr(J.err, 2);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      uint32_t it = 0, f = 0;
      for (int64_t t = blockIdx.x; t < J.n_tiles && !abort_flag; t += gridDim.x) {
        OzTile T;
        oz_decode(J, t, T);
        const uint32_t idesc = idesc_bf16_f32(OZ_M, (uint32_t)T.nmma);
        int kc = 0;
        for (int64_t sidx = T.seg0; sidx < T.seg1 && !abort_flag; sidx++) {
          const int64_t p = J.g.perm ? J.g.perm[sidx] : sidx;
          const int64_t nk = J.nk_pair[p];
          for (int64_t q = 0; q < nk; q++, it++) {
            const uint32_t st = it % NS, use = it / NS;
            if (!mbar_wait(&full_bar[st], use & 1)) {
              atomicOr(J.err, 4);
              abort_flag = 1;
              break;
            }
            tc_fence_after();
            if (kc == 0) {
              if (f > 0 && !mbar_wait(&acc_empty, (f - 1) & 1)) {
                atomicOr(J.err, 8);
                abort_flag = 1;
                break;
              }
              tc_fence_after();
            }
            const uint32_t sa = smem_u32(smem + st * stage_bytes);
            oz_issue_s(s, tmem, smem_desc(sa, 128, 256), smem_desc(sa + a_bytes_max, 128, 256),
                       (uint32_t)T.ga * 16, (uint32_t)T.gb * 16, idesc, kc == 0);
            mma_commit(&empty_bar[st]);
            if (++kc == OZ_CHUNK) {
              mma_commit(&acc_full);
              f++;
              kc = 0;
            }
          }
        }
        if (kc > 0 && !abort_flag) {
          mma_commit(&acc_full);
          f++;
        }
      }
      // every MMA issued must finish before TMEM is released
      mma_commit(&done_bar);
      if (!mbar_wait(&done_bar, 0)) atomicOr(J.err, 32);
    }
  } else {
    // ---------------- epilogue: 8 warps; warp -> TMEM lane quarter, column half
    const int q4 = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row = 32 * q4 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q4) << 16);
    const int cbase = half * (OZ_N / 2);
    const int n_acc = s < OZ_NACC ? s : OZ_NACC;  // accumulators the slice products reach
    uint32_t f = 0;
    for (int64_t t = blockIdx.x; t < J.n_tiles && !abort_flag; t += gridDim.x) {
      OzTile T;
      oz_decode(J, t, T);
      const int64_t nflush = (T.ksum + OZ_CHUNK - 1) / OZ_CHUNK;
      const int64_t grow = T.mt * OZ_M + row;
      const bool row_ok = grow < T.m;
      const int er = row_ok ? J.expA[J.rowA[J.keyA[T.i0]] + grow] : 0;
      // S: running sum in units of 2^-u of the leading slice product.  With
      // u <= 48 - log2(K) the sum stays below 2^62.1 for any data, and u >= 24
      // keeps D0..D3 (whole multiples of 2^-24) exact.
      int kb = 0;
      while (kb < 40 && (int64_t(1) << kb) < 16 * T.ksum) kb++;
      const int u = 48 - kb < 32 ? 48 - kb : 32;
      // D_a (a < 4) holds multiples of 2^-8a below 2^24 * 2^-8a: D_a 2^8a is a
      // whole number of int32; D4 is rounded at 2^-u
      float scale[OZ_NACC];
      int shift[OZ_NACC];
#pragma unroll
      for (int a = 0; a < OZ_NACC - 1; a++) {
        scale[a] = __int_as_float((127 + 8 * a) << 23);
        shift[a] = u - 8 * a;
      }
      scale[OZ_NACC - 1] = __int_as_float((127 + u) << 23);
      shift[OZ_NACC - 1] = 0;
      long long S[OZ_N / 2];
#pragma unroll
      for (int y = 0; y < OZ_N / 2; y++) S[y] = 0;
      for (int64_t c = 0; c < nflush; c++, f++) {
        if (!mbar_wait(&acc_full, f & 1)) {
          atomicOr(J.err, 16);
          abort_flag = 1;
          break;
        }
        tc_fence_after();
        // one 8-column chunk of every accumulator per round, a single wait
#pragma unroll
        for (int x = 0; x < OZ_N / 16; x++) {
          uint32_t v[OZ_NACC][8];
#pragma unroll
          for (int a = 0; a < OZ_NACC; a++)
            if (a < n_acc) tmem_ld8(lane_addr + a * OZ_N + cbase + 8 * x, v[a]);
          tmem_ld_wait();
#pragma unroll
          for (int a = 0; a < OZ_NACC; a++) {
            if (a >= n_acc) break;
#pragma unroll
            for (int y = 0; y < 8; y++)
              S[8 * x + y] += (long long)oz_to_int(__uint_as_float(v[a][y]), scale[a]) << shift[a];
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty);
      }
      if (abort_flag) break;
      // C = S * 2^(e_r + f_c - 16 - u)
      double *C = (double *)J.g.C + J.g.c_off[T.o];
      const int64_t *rowB = J.rowB + J.keyB[T.j0];
      if (row_ok) {
#pragma unroll
        for (int y = 0; y < OZ_N / 2; y++) {
          const int64_t gcol = T.nt * OZ_N + cbase + y;
          if (gcol < T.n) {
            const int fc = J.expB[*rowB + gcol];
            C[grow + gcol * T.m] = oz_i64_ldexp(S[y], er + fc - 16 - u);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, OZ_TMEM_COLS);
  }
}

// ---------------------------------------------------------------- host side
int oz_stages(int s) {
  const int stage = s * ((OZ_M + OZ_N) / 8) * 256;
  int n = OZ_SMEM_BYTES / stage;
  return n > OZ_MAX_STAGES ? OZ_MAX_STAGES : n;
}

tq_status launch_ozaki_prepare(const OzJob &job, const OzSide &SA, const OzSide &SB,
                               int64_t rowsA, int64_t rowsB, int64_t tilesA, int64_t tilesB,
                               int32_t *expA, int32_t *expB, int64_t nexpA, int64_t nexpB,
                               cudaStream_t st) {
  const int T = 256;
  if (nexpA) count_launch(), oz_exp_init_kernel<<<(unsigned)((nexpA + T - 1) / T), T, 0, st>>>(expA, nexpA);
  if (nexpB) count_launch(), oz_exp_init_kernel<<<(unsigned)((nexpB + T - 1) / T), T, 0, st>>>(expB, nexpB);
  if (rowsA) count_launch(), oz_rowexp_kernel<<<(unsigned)((rowsA + T - 1) / T), T, 0, st>>>(SA, rowsA, expA);
  if (rowsB) count_launch(), oz_rowexp_kernel<<<(unsigned)((rowsB + T - 1) / T), T, 0, st>>>(SB, rowsB, expB);
  TQ_CUDA(cudaGetLastError());
  if (tilesA) count_launch(), oz_slice_kernel<<<(unsigned)tilesA, 256, 0, st>>>(SA, job.s, OZ_M, expA,
                                                                  (uint8_t *)job.sliceA);
  if (tilesB) count_launch(), oz_slice_kernel<<<(unsigned)tilesB, 256, 0, st>>>(SB, job.s, OZ_N, expB,
                                                                  (uint8_t *)job.sliceB);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

tq_status launch_ozaki_gemm(const OzJob &job, cudaStream_t st) {
  if (job.n_tiles == 0) return TQ_OK;
  static int sms = 0;
  if (!sms) {
    int dev;
    TQ_CUDA(cudaGetDevice(&dev));
    TQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TQ_CUDA(cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 OZ_SMEM_BYTES));
  }
  const int64_t grid = job.n_tiles < sms ? job.n_tiles : sms;
  count_launch(), oz_gemm_kernel<<<(unsigned)grid, OZ_THREADS, OZ_SMEM_BYTES, st>>>(job);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

}  // namespace tq
