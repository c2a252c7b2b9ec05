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
//     fp32 accumulation in TMEM, in four accumulators by g = t+u: D0..D2
//     (g = 0..2) hold multiples of 2^(-8g) below (g+1) K 2^14 2^(-8g), whole
//     numbers of 24 bits or fewer for K <= 336, so the tensor core sums them
//     exactly; D3 (g >= 3, at most 2^-24 of D0) is rounded.  Each accumulator is
//     retired after at most 336 columns of the fused K (all pairs of the output
//     block, in order) on a staggered schedule and restarted in a spare TMEM
//     slot, while the epilogue folds the retired slot into an int64 running sum
//     S = sum round(2^u D_a) held in registers (u per tile, so no data can
//     overflow it) — the MMAs do not wait for the fold.  A single fp32
//     accumulator for the lower groups is not enough: the tensor core's fp32
//     accumulation truncates, which loses about K ulps of the group it holds.
//   * C = S * 2^(e_r + f_c - 16 - u), converted to FP64 with integer operations.
// No FP64 arithmetic runs in the GEMM: GB300 issues about 2 FP64 FMAs per SM
// per clock against ~4000 bf16 FMAs, so FP64 work stays in the row-exponent
// pass (one ilogb per row) only.
//
// Layout of the sliced operands in global memory (built by oz_slice_kernel):
// for every operand block, row tiles of RT rows (128 for A, the tile width 32,
// 64 or 96 for B); in a
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
// TMEM: OZ_NACC + 1 slots of tile-width columns (at most 480 of 512)
constexpr int OZ_NACC = 4;
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

__device__ __forceinline__ void side_operand(const OzSide &S, int64_t b, Operand &op) {
  int64_t cb[TQ_MAXR], ce[TQ_MAXR];
  for (int k = 0; k < S.ncon; k++) {
    cb[k] = S.T.begin[b * S.T.rank + S.con[k]];
    ce[k] = S.T.end[b * S.T.rank + S.con[k]];
  }
  build_operand(S.T, b, S.nfree, S.free_legs, S.ncon, S.con, cb, ce, op);
}

// ---------------------------------------------------------------- exponents
__global__ void oz_exp_init_kernel(OzLaunch L) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= L.n_exps) return;
  const int64_t k = oz_find(L.side_exp_start, L.n_sides, g);
  L.sides[k].exps[g - L.side_exp_start[k]] = OZ_EXP_ZERO;
}

// One thread per (side, block, row): max |x| over the row's contracted columns.
__global__ void oz_rowexp_kernel(OzLaunch L) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= L.n_rows) return;
  const int64_t k = oz_find(L.side_row_start, L.n_sides, g);
  const OzSide &S = L.sides[k];
  const int64_t lr = g - L.side_row_start[k];
  const int64_t b = oz_find(S.row_start, S.T.nb, lr);
  const int64_t r = lr - S.row_start[b];
  Operand op;
  side_operand(S, b, op);
  const double *d = (const double *)S.T.data;
  const int64_t ra = op.base + mixed_addr(r, op.nr, op.rdim, op.rst);
  unsigned long long mx = 0;
  for (int64_t c = 0; c < op.cols; c++) {
    const unsigned long long bits =
        (unsigned long long)__double_as_longlong(d[ra + mixed_addr(c, op.nc, op.cdim, op.cst)]) &
        0x7fffffffffffffffull;
    mx = bits > mx ? bits : mx;
  }
  if (mx == 0) return;
  const int e = ilogb(__longlong_as_double((long long)mx)) + 2;
  atomicMax(&S.exps[S.row_off[S.key[b]] + r], e);
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

// The s slices of k-step q for one half row (8 columns, c = 0 or 1) of row r of
// an operand row tile with G row groups, written into the k-step's chunk.
__device__ __forceinline__ void oz_slice_kstep(const double *d, bool row_ok, int64_t ra,
                                               const Operand &op, int64_t q, int c, int shift,
                                               int s, int G, int r, uint8_t *chunk) {
  uint32_t packed[OZ_MAXS][4];
#pragma unroll
  for (int t = 0; t < OZ_MAXS; t++)
#pragma unroll
    for (int w = 0; w < 4; w++) packed[t][w] = 0;
#pragma unroll
  for (int x = 0; x < 8; x++) {
    const int64_t kk = q * 16 + c * 8 + x;
    long long F = 0;
    if (row_ok && kk < op.cols) F = oz_fixed(d[ra + mixed_addr(kk, op.nc, op.cdim, op.cst)], shift);
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

// Class layout: one work item is a row tile of a class times one of its
// contracted boxes; the tile's rows come from the blocks of several free boxes.
__device__ __forceinline__ void oz_slice_class(const OzSide &S, int64_t lt) {
  const OzClassItem it = S.items[lt];
  const int s = S.s;
  const int G = (it.rows + 7) / 8;
  const int r = threadIdx.x >> 1, c = threadIdx.x & 1;
  if (r >= G * 8) return;
  const bool row_ok = r < it.rows;
  Operand op;
  op.cols = 0;
  op.nc = 0;
  int64_t ra = 0;
  int e = OZ_EXP_ZERO;
  if (row_ok) {
    const int64_t vr = it.vrow0 + r;
    const OzRowMap rm = S.rmap[vr];
    const int64_t b = S.blk[it.blk_base + (int64_t)rm.xi * it.nbox + it.box];
    side_operand(S, b, op);
    ra = op.base + mixed_addr(rm.xr, op.nr, op.rdim, op.rst);
    e = S.exps[vr];
  }
  uint8_t *base = S.slices + 256 * it.unit + (int64_t)it.koff * s * G * 256;
  const double *d = (const double *)S.T.data;
  for (int64_t q = 0; q < it.nk; q++)
    oz_slice_kstep(d, row_ok, ra, op, q, c, 8 * s - e, s, G, r, base + q * (int64_t)s * G * 256);
}

// One CTA per (side, block, row tile): slices of all k-steps of the tile (or,
// for a side in the class layout, one CTA per work item).
__global__ void __launch_bounds__(256) oz_slice_kernel(OzLaunch L) {
  const int64_t g = blockIdx.x;
  const int64_t k = oz_find(L.side_tile_start, L.n_sides, g);
  const OzSide &S = L.sides[k];
  const int64_t lt = g - L.side_tile_start[k];
  if (S.items) {
    oz_slice_class(S, lt);
    return;
  }
  const int64_t b = oz_find(S.tile_start, S.T.nb, lt);
  const int64_t rt = lt - S.tile_start[b];
  const int s = S.s, rt_rows = S.rt_rows;
  Operand op;
  side_operand(S, b, op);
  const int64_t rows = op.rows - rt * rt_rows < rt_rows ? op.rows - rt * rt_rows : rt_rows;
  const int G = (int)((rows + 7) / 8);
  const int64_t nk = (op.cols + 15) / 16;
  uint8_t *base = S.slices + 256 * S.unit_off[b] + nk * (int64_t)s * 256 * (rt_rows / 8) * rt;
  const double *d = (const double *)S.T.data;
  const int r = threadIdx.x >> 1, c = threadIdx.x & 1;
  if (r >= G * 8) return;
  const int64_t grow = rt * rt_rows + r;
  const bool row_ok = r < rows;
  const int e = row_ok ? S.exps[S.row_off[S.key[b]] + grow] : OZ_EXP_ZERO;
  const int64_t ra = row_ok ? op.base + mixed_addr(grow, op.nr, op.rdim, op.rst) : 0;
  for (int64_t q = 0; q < nk; q++)
    oz_slice_kstep(d, row_ok, ra, op, q, c, 8 * s - e, s, G, r, base + q * (int64_t)s * G * 256);
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
// Accumulators by g = t+u: D0, D1, D2 (exact) and D3 (g >= 3, rounded).  They
// live in TMEM slots of tile-width columns, more slots than accumulators (five
// for width 96, eight for 32 and 64): accumulator a is retired after every
// OZ_CHUNK k-steps on its own staggered schedule (first after
// OZ_CHUNK - OZ_STAG*a), and at the end of its tile; it then restarts in the
// free slot retired longest ago, and the retired slot is drained by the
// epilogue while the MMAs go on.  With eight slots a whole tile's accumulators
// move to fresh slots at its end, so the next tile's MMAs start before the
// epilogue has drained the last one.  Each slot has its own full/empty barrier
// pair, so no parity wait can fall two phases behind: a slot is never retired
// twice without a drain in between.
constexpr int OZ_MAXSLOT = 2 * OZ_NACC;
constexpr int OZ_STAG = 5;
constexpr int OZ_FINAL = 100;
template <int N>
struct OzSlots {
  static constexpr int n = N <= 32 ? 2 * OZ_NACC : N <= 64 ? 2 * OZ_NACC - 1 : OZ_NACC + 1;
  static_assert(n * N <= (int)OZ_TMEM_COLS, "slots exceed TMEM");
  // A slices held in tensor memory after the slots (8 columns each)
  static constexpr int ntm = ((int)OZ_TMEM_COLS - n * N) / 8;
};
static_assert(OZ_STAG * (OZ_NACC - 1) < OZ_CHUNK, "stagger must fit one chunk");

// All slice products of one k-step, fully unrolled: product (t, u) goes to
// accumulator min(t+u, OZ_NACC-1) at TMEM column slot[acc].  Descriptors advance
// by whole row groups (the start-address field counts 16-byte units).  The first
// product of the k-step into an accumulator whose bit is set in `fresh`
// overwrites it.  A slices t < NTM are copied once into tensor memory (columns
// acol + 8t) and their products read them there: each A slice is used by up to s
// products, and reading it from shared memory for every one of them would take
// most of the shared-memory bandwidth the tensor core has (128 B per clock).
// The copies are ordered before the MMAs of the same thread, and the MMAs of a
// k-step before the next k-step's copies.
template <int S, bool FRESH, int NTM>
__device__ __forceinline__ void oz_issue(const uint32_t (&col)[OZ_NACC], uint64_t da0,
                                         uint64_t db0, uint32_t a_step, uint32_t b_step,
                                         uint32_t idesc, uint32_t fresh, uint32_t acol) {
#pragma unroll
  for (int t = 0; t < S && t < NTM; t++)
    tmem_cp_128x256b(acol + 8 * t, da0 + (uint64_t)(t * a_step));
#pragma unroll
  for (int t = 0; t < S; t++) {
#pragma unroll
    for (int u = 0; u < S - t; u++) {
      const int acc = t + u < OZ_NACC - 1 ? t + u : OZ_NACC - 1;
      // first (t, u) in this order that lands in accumulator acc
      const bool first = acc < OZ_NACC - 1 ? t == 0 : (t == 0 && u == OZ_NACC - 1);
      const uint32_t keep = (FRESH && first && ((fresh >> acc) & 1)) ? 0u : 1u;
      if (t < NTM)
        mma_bf16_ta(col[acc], acol + 8 * t, db0 + (uint64_t)(u * b_step), idesc, keep);
      else
        mma_bf16(col[acc], da0 + (uint64_t)(t * a_step), db0 + (uint64_t)(u * b_step), idesc,
                 keep);
    }
  }
}

template <bool FRESH, int NTM>
__device__ __forceinline__ void oz_issue_s(int s, const uint32_t (&col)[OZ_NACC], uint64_t da0,
                                           uint64_t db0, uint32_t a_step, uint32_t b_step,
                                           uint32_t idesc, uint32_t fresh, uint32_t acol) {
  switch (s) {
    case 1: oz_issue<1, FRESH, NTM>(col, da0, db0, a_step, b_step, idesc, fresh, acol); break;
    case 2: oz_issue<2, FRESH, NTM>(col, da0, db0, a_step, b_step, idesc, fresh, acol); break;
    case 3: oz_issue<3, FRESH, NTM>(col, da0, db0, a_step, b_step, idesc, fresh, acol); break;
    case 4: oz_issue<4, FRESH, NTM>(col, da0, db0, a_step, b_step, idesc, fresh, acol); break;
    case 5: oz_issue<5, FRESH, NTM>(col, da0, db0, a_step, b_step, idesc, fresh, acol); break;
    case 6: oz_issue<6, FRESH, NTM>(col, da0, db0, a_step, b_step, idesc, fresh, acol); break;
    default: oz_issue<7, FRESH, NTM>(col, da0, db0, a_step, b_step, idesc, fresh, acol); break;
  }
}

// Retirement schedule of a tile with ksum k-steps: next event after k-step k.
// Returns the k-step (1-based) of the next event and its kind (accumulator
// index, or OZ_FINAL at the end of the tile, which retires every accumulator).
struct OzSchedule {
  int64_t next[OZ_NACC];
  int64_t ksum;
  int n_acc;
  __device__ __forceinline__ void start(int64_t ks, int na) {
    ksum = ks;
    n_acc = na;
#pragma unroll
    for (int a = 0; a < OZ_NACC; a++) next[a] = OZ_CHUNK - OZ_STAG * a;
  }
  // event at or after the current position: (k, kind)
  __device__ __forceinline__ void peek(int64_t &k, int &kind) const {
    k = ksum;
    kind = OZ_FINAL;
#pragma unroll
    for (int a = 0; a < OZ_NACC; a++)
      if (a < n_acc && next[a] < k) {
        k = next[a];
        kind = a;
      }
  }
  __device__ __forceinline__ void advance(int kind) {
    if (kind != OZ_FINAL) next[kind] += OZ_CHUNK;
  }
};

// Which TMEM slot each accumulator occupies, replayed identically by the three
// roles of the GEMM: accumulator a sits in slot bits [3a, 3a+3) of `map`; the
// free slots wait in `fifo` (3 bits each, oldest retirement first); per slot p,
// bit p of `par` is the parity of its retirements so far and bit p of `used`
// whether it had one.
template <int NSLOT>
struct OzSlotMap {
  static constexpr int NFREE = NSLOT - OZ_NACC;
  uint32_t map, par, used, fifo;
  __device__ __forceinline__ void init() {
    map = par = used = fifo = 0;
#pragma unroll
    for (int a = 0; a < OZ_NACC; a++) map |= (uint32_t)a << (3 * a);
#pragma unroll
    for (int q = 0; q < NFREE; q++) fifo |= (uint32_t)(OZ_NACC + q) << (3 * q);
  }
  __device__ __forceinline__ uint32_t slot(int a) const { return (map >> (3 * a)) & 7; }
  // accumulator a leaves its slot (returned) and restarts in the oldest free one
  __device__ __forceinline__ uint32_t retire(int a) {
    const uint32_t p = slot(a);
    par ^= 1u << p;
    used |= 1u << p;
    const uint32_t q = fifo & 7;
    fifo = (fifo >> 3) | (p << (3 * (NFREE - 1)));
    map = (map & ~(7u << (3 * a))) | (q << (3 * a));
    return p;
  }
  // parity of the drain that must complete before slot p is written again
  __device__ __forceinline__ bool needs_drain(uint32_t p) const { return (used >> p) & 1; }
  __device__ __forceinline__ uint32_t drain_parity(uint32_t p) const { return ((par >> p) & 1) ^ 1; }
};

// Exact fp32 -> int32 for values whose scaled magnitude is below 2^22 (one FMA
// against 1.5 * 2^23, whose ulp is 1, then an integer subtract; rounds to
// nearest even like rint); larger values take the conversion unit.
__device__ __forceinline__ int oz_to_int(float x, float scale) {
  const float y = x * scale;
  if (fabsf(y) < 4194304.0f) return __float_as_int(y + 12582912.0f) - 0x4B400000;
  return __float2int_rn(y);
}

struct OzTile {
  const OzJob *J;
  int64_t o, mt, nt, m, n, i0, j0, seg0, seg1, ksum, c_off, erow, ecol;
  int32_t ga, gb, nmma;
};

// Global tile t of the launch -> its job and (output block, row tile, column tile).
template <int N>
__device__ __forceinline__ void oz_decode(const OzLaunch &L, int64_t t, OzTile &T) {
  const int64_t j = oz_find(L.job_tile_start, L.n_jobs, t);
  const OzJob &J = L.jobs[j];
  T.J = &J;
  t -= L.job_tile_start[j];
  if (J.cls) {
    // class layout: output = class, one pseudo-pair per class
    T.o = oz_find(J.tile_start, J.n_cls, t);
    const OzClassOut K = J.cls[T.o];
    T.seg0 = T.o;
    T.seg1 = T.o + 1;
    T.i0 = T.j0 = 0;
    T.m = K.m;
    T.n = K.n;
  } else {
    T.o = oz_find(J.tile_start, J.g.n_out, t);
    T.seg0 = J.g.seg[T.o];
    T.seg1 = J.g.seg[T.o + 1];
    const int64_t p0 = J.g.perm ? J.g.perm[T.seg0] : T.seg0;
    T.i0 = J.g.pa[p0];
    T.j0 = J.g.pb[p0];
    T.m = free_rows(J.g.A, T.i0, J.g.L.nfa, J.g.L.fa);
    T.n = free_rows(J.g.B, T.j0, J.g.L.nfb, J.g.L.fb);
  }
  // tiles in bands of OZ_BAND row tiles, column tiles in order within a band:
  // the CTAs working at the same time (consecutive tiles) then share a few row
  // tiles' A operands and a band's worth of B operands in L2, instead of
  // streaming one column tile against every row tile of a tall output
  const int64_t tiles_m = (T.m + OZ_M - 1) / OZ_M;
  const int64_t tiles_n = (T.n + N - 1) / N;
  const int64_t local = t - J.tile_start[T.o];
  const int64_t band = local / (OZ_BAND * tiles_n);
  const int64_t band_rows = min((int64_t)OZ_BAND, tiles_m - band * OZ_BAND);
  const int64_t in_band = local - band * OZ_BAND * tiles_n;
  T.nt = in_band / band_rows;
  T.mt = band * OZ_BAND + in_band % band_rows;
  const int64_t ra = min((int64_t)OZ_M, T.m - T.mt * OZ_M);
  const int64_t rb = min((int64_t)N, T.n - T.nt * N);
  T.ga = (int32_t)((ra + 7) / 8);
  T.gb = (int32_t)((rb + 7) / 8);
  T.nmma = (int32_t)(16 * ((rb + 15) / 16));
  T.ksum = J.ksum[T.o];
}

// The tile table of a launch (built once per batch).
template <int N>
__global__ void oz_table_kernel(OzLaunch L, OzTileRec *out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= L.n_tiles) return;
  OzTile T;
  oz_decode<N>(L, t, T);
  const OzJob &J = *T.J;
  OzTileRec r;
  r.seg0 = T.seg0;
  r.seg1 = T.seg1;
  r.ksum = T.ksum;
  r.c_off = J.cls ? 0 : J.g.c_off[T.o];
  r.m = T.m;
  r.n = T.n;
  r.erow = J.cls ? J.cls[T.o].erow : J.rowA[J.keyA[T.i0]];
  r.ecol = J.cls ? J.cls[T.o].ecol : J.rowB[J.keyB[T.j0]];
  r.job = (int32_t)(T.J - L.jobs);
  r.mt = (int32_t)T.mt;
  r.nt = (int32_t)T.nt;
  r.packed = T.ga | (T.gb << 8) | (T.nmma << 16);
  out[t] = r;
}

// The pair table of one job (built when its plan is made).
__global__ void oz_pair_table_kernel(const int64_t *perm, const int32_t *pa, const int32_t *pb,
                                     const int64_t *unitA, const int64_t *unitB,
                                     const int32_t *nk_pair, int64_t n, OzPairRec *out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int64_t p = perm ? perm[q] : q;
  OzPairRec r;
  r.a_off = 256 * unitA[pa[p]];
  r.b_off = 256 * unitB[pb[p]];
  r.nk = nk_pair[p];
  r.pad = 0;
  out[q] = r;
}

tq_status oz_pair_table(const OzJob &J, int64_t n_pairs, OzPairRec *out, cudaStream_t st) {
  if (n_pairs == 0) return TQ_OK;
  count_launch(), oz_pair_table_kernel<<<(unsigned)((n_pairs + 255) / 256), 256, 0, st>>>(
      J.g.perm, J.g.pa, J.g.pb, J.unitA, J.unitB, J.nk_pair, n_pairs, out);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

__device__ __forceinline__ void oz_unpack(const OzLaunch &L, const OzTileRec &r, OzTile &T) {
  T.J = L.jobs + r.job;
  T.seg0 = r.seg0;
  T.seg1 = r.seg1;
  T.ksum = r.ksum;
  T.c_off = r.c_off;
  T.m = r.m;
  T.n = r.n;
  T.erow = r.erow;
  T.ecol = r.ecol;
  T.mt = r.mt;
  T.nt = r.nt;
  T.ga = r.packed & 0xff;
  T.gb = (r.packed >> 8) & 0xff;
  T.nmma = r.packed >> 16;
}

template <int N>
__global__ void __launch_bounds__(OZ_THREADS, 1) oz_gemm_kernel(OzLaunch L) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full_bar[OZ_MAX_STAGES], empty_bar[OZ_MAX_STAGES];
  __shared__ __align__(8) uint64_t slot_full[OZ_MAXSLOT], slot_empty[OZ_MAXSLOT], done_bar;
  constexpr int NSLOT = OzSlots<N>::n;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int NS = L.nstages;
  // stages are sized for the largest slice count of the batch
  const uint32_t a_bytes_max = (uint32_t)L.s_max * (OZ_M / 8) * 256;
  const uint32_t stage_bytes = (uint32_t)L.s_max * ((OZ_M + N) / 8) * 256;

  if (threadIdx.x == 0) {
    for (int q = 0; q < NS; q++) {
      mbar_init(&full_bar[q], 1);
      mbar_init(&empty_bar[q], 1);
    }
    for (int q = 0; q < NSLOT; q++) {
      mbar_init(&slot_full[q], 1);
      mbar_init(&slot_empty[q], 8);
    }
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
    // ---------------- producer: one bulk copy per operand per k-step.  It also
    // replays the accumulator schedule and, before filling a stage whose MMAs
    // restart accumulators in TMEM slots used before, waits until the epilogue
    // has drained those slots: the MMA warp then only waits for its stage (the
    // stage's completion implies the drain) and keeps feeding the tensor core.
    if (lane == 0) {
      OzSlotMap<NSLOT> sm;
      sm.init();
      uint32_t it = 0;
      // stage of k-step `it` and the parity of its previous use (counters, not it % NS)
      uint32_t st = 0, ph = 1;
      // the next tile's record is loaded one tile ahead
      OzTileRec nxt;
      if (blockIdx.x < L.n_tiles) nxt = L.tiles[blockIdx.x];
      for (int64_t t = blockIdx.x; t < L.n_tiles && !abort_flag; t += gridDim.x) {
        const OzTileRec cur = nxt;
        if (t + gridDim.x < L.n_tiles) nxt = L.tiles[t + gridDim.x];
        OzTile T;
        oz_unpack(L, cur, T);
        // job fields in registers: the asm memory clobbers below would reload them
        const OzJob &J = *T.J;
        const int s = J.s;
        const OzPairRec *prs = J.prs;
        const uint8_t *sliceA = J.sliceA, *sliceB = J.sliceB;
        const uint32_t ba = (uint32_t)s * T.ga * 256, bb = (uint32_t)s * T.gb * 256;
        const int n_acc = s < OZ_NACC ? s : OZ_NACC;
        OzSchedule sch;
        sch.start(T.ksum, n_acc);
        int64_t ev_k;
        int ev_kind;
        sch.peek(ev_k, ev_kind);
        uint32_t fresh = (1u << n_acc) - 1;
        int64_t k = 0;
        // the next pair's record is loaded one pair ahead
        OzPairRec pn = prs[T.seg0];
        for (int64_t sidx = T.seg0; sidx < T.seg1 && !abort_flag; sidx++) {
          const OzPairRec pr = pn;
          if (sidx + 1 < T.seg1) pn = prs[sidx + 1];
          const int64_t nk = pr.nk;
          const uint8_t *ga = sliceA + pr.a_off + nk * s * 256 * (OZ_M / 8) * T.mt;
          const uint8_t *gb = sliceB + pr.b_off + nk * s * 256 * (N / 8) * T.nt;
          for (int64_t q = 0; q < nk; q++, it++) {
            if (it >= (uint32_t)NS && !mbar_wait(&empty_bar[st], ph)) {
              atomicOr(L.err, 1);
              abort_flag = 1;
              break;
            }
            if (fresh) {
              bool ok = true;
#pragma unroll
              for (int a = 0; a < OZ_NACC; a++) {
                const uint32_t p = sm.slot(a);
                if (((fresh >> a) & 1) && sm.needs_drain(p) &&
                    !mbar_wait(&slot_empty[p], sm.drain_parity(p)))
                  ok = false;
              }
              if (!ok) {
                atomicOr(L.err, 8);
                abort_flag = 1;
                break;
              }
              fresh = 0;
            }
            uint8_t *sa = smem + st * stage_bytes;
            mbar_arrive_expect_tx(&full_bar[st], ba + bb);
            bulk_g2s(sa, ga + q * ba, ba, &full_bar[st]);
            bulk_g2s(sa + a_bytes_max, gb + q * bb, bb, &full_bar[st]);
            if (++st == (uint32_t)NS) {
              st = 0;
              ph ^= 1;
            }
            if (++k == ev_k) {
#pragma unroll
              for (int a = 0; a < OZ_NACC; a++) {
                if (a >= n_acc || (ev_kind != OZ_FINAL && a != ev_kind)) continue;
                sm.retire(a);
                fresh |= 1u << a;
              }
              if (ev_kind != OZ_FINAL) {
                sch.advance(ev_kind);
                sch.peek(ev_k, ev_kind);
              }
            }
          }
        }
      }
      // drain: every copy issued must land before the CTA may exit
      const uint32_t first = it > (uint32_t)NS ? it - NS : 0;
      for (uint32_t q = first; q < it; q++) {
        if (!mbar_wait(&full_bar[q % NS], (q / NS) & 1)) atomicOr(L.err, 2);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer.  The whole warp runs the loop, so the MMA
    // operands are warp-uniform values; lane 0 waits on the barriers and one
    // elected lane (the same one throughout) issues the copies, MMAs and commits.
    {
      constexpr uint32_t FULL = 0xffffffffu;
      uint32_t it = 0;
      uint32_t st = 0, ph = 0;  // stage of k-step `it` and its fill parity
      // smem descriptors of stage 0; a stage's are these plus its offset / 16
      const uint32_t sm0 = smem_u32(smem);
      const uint64_t dA0 = smem_desc(sm0, 128, 256), dB0 = smem_desc(sm0 + a_bytes_max, 128, 256);
      OzSlotMap<NSLOT> sm;
      sm.init();
      // the next tile's record is loaded one tile ahead
      OzTileRec nxt;
      if (blockIdx.x < L.n_tiles) nxt = L.tiles[blockIdx.x];
      for (int64_t t = blockIdx.x; t < L.n_tiles && !__shfl_sync(FULL, abort_flag, 0);
           t += gridDim.x) {
        const OzTileRec cur = nxt;
        if (t + gridDim.x < L.n_tiles) nxt = L.tiles[t + gridDim.x];
        OzTile T;
        oz_unpack(L, cur, T);
        const OzJob &J = *T.J;
        const int s = J.s;
        const int n_acc = s < OZ_NACC ? s : OZ_NACC;
        const OzPairRec *prs = J.prs;
        const uint32_t idesc = idesc_bf16_f32(OZ_M, (uint32_t)T.nmma);
        OzSchedule sch;
        sch.start(T.ksum, n_acc);
        int64_t ev_k;
        int ev_kind;
        sch.peek(ev_k, ev_kind);
        uint32_t fresh = (1u << n_acc) - 1;  // accumulators to (re)start in a free slot
        int64_t k = 0;
        uint32_t col[OZ_NACC];
#pragma unroll
        for (int a = 0; a < OZ_NACC; a++) col[a] = tmem + sm.slot(a) * N;
        int32_t nk_next = prs[T.seg0].nk;
        for (int64_t sidx = T.seg0; sidx < T.seg1 && !__shfl_sync(FULL, abort_flag, 0); sidx++) {
          const int64_t nk = nk_next;
          if (sidx + 1 < T.seg1) nk_next = prs[sidx + 1].nk;
          for (int64_t q = 0; q < nk; q++, it++) {
            int ok = 1;
            if (lane == 0) ok = mbar_wait(&full_bar[st], ph);
            if (!__shfl_sync(FULL, ok, 0)) {
              if (lane == 0) {
                atomicOr(L.err, 4);
                abort_flag = 1;
              }
              break;
            }
            tc_fence_after();
            const uint64_t so = (uint64_t)((st * stage_bytes) >> 4);
            if (elect_one()) {
              oz_issue_s<true, OzSlots<N>::ntm>(s, col, dA0 + so, dB0 + so, (uint32_t)T.ga * 16,
                                                (uint32_t)T.gb * 16, idesc, fresh,
                                                tmem + NSLOT * N);
              mma_commit(&empty_bar[st]);
            }
            __syncwarp();
            if (++st == (uint32_t)NS) {
              st = 0;
              ph ^= 1;
            }
            fresh = 0;
            if (++k == ev_k) {
#pragma unroll
              for (int a = 0; a < OZ_NACC; a++) {
                if (a >= n_acc || (ev_kind != OZ_FINAL && a != ev_kind)) continue;
                const uint32_t p = sm.slot(a);
                if (elect_one()) mma_commit(&slot_full[p]);
                __syncwarp();
                sm.retire(a);
                col[a] = tmem + sm.slot(a) * N;
                fresh |= 1u << a;
              }
              if (ev_kind != OZ_FINAL) {
                sch.advance(ev_kind);
                sch.peek(ev_k, ev_kind);
              }
            }
          }
        }
      }
      // every MMA issued must finish before TMEM is released
      if (elect_one()) mma_commit(&done_bar);
      __syncwarp();
      if (lane == 0 && !mbar_wait(&done_bar, 0)) atomicOr(L.err, 32);
    }
  } else {
    // ---------------- epilogue: 8 warps; warp -> TMEM lane quarter, column half
    const int q4 = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row = 32 * q4 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q4) << 16);
    const int cbase = half * (N / 2);
    // the MMA warp's slot map, replayed
    OzSlotMap<NSLOT> sm;
    sm.init();
    for (int64_t t = blockIdx.x; t < L.n_tiles && !abort_flag; t += gridDim.x) {
      OzTile T;
      oz_unpack(L, L.tiles[t], T);
      const OzJob &J = *T.J;
      const int n_acc = J.s < OZ_NACC ? J.s : OZ_NACC;
      const int64_t grow = T.mt * OZ_M + row;
      const bool row_ok = grow < T.m;
      const int er = row_ok ? J.expA[T.erow + grow] : 0;
      // S: running sum in units of 2^-u of the leading slice product.  With
      // u <= 48 - log2(K) the sum stays below 2^62.1 for any data, and u >= 24
      // keeps D0..D2 (whole multiples of 2^-16) exact.
      int kb = 0;
      while (kb < 40 && (int64_t(1) << kb) < 16 * T.ksum) kb++;
      const int u = 48 - kb < 32 ? 48 - kb : 32;
      long long S[N / 2];
#pragma unroll
      for (int y = 0; y < N / 2; y++) S[y] = 0;
      OzSchedule sch;
      sch.start(T.ksum, n_acc);
      bool done = false;
      while (!done && !abort_flag) {
        int64_t ev_k;
        int ev_kind;
        sch.peek(ev_k, ev_kind);
        done = ev_kind == OZ_FINAL;
        // drain the retired slot(s): D_a (a < 3) holds multiples of 2^-8a below
        // 2^24 * 2^-8a, so D_a 2^8a is a whole int32; D3 is rounded at 2^-u
#pragma unroll
        for (int a = 0; a < OZ_NACC; a++) {
          if (a >= n_acc || (!done && a != ev_kind)) continue;
          const uint32_t p = sm.slot(a);
          // the retirement being drained is the (par_p + 1)-th of slot p
          if (!mbar_wait(&slot_full[p], ((sm.par >> p) & 1))) {
            atomicOr(L.err, 16);
            abort_flag = 1;
            break;
          }
          tc_fence_after();
          const float scale = a < OZ_NACC - 1 ? __int_as_float((127 + 8 * a) << 23)
                                              : __int_as_float((127 + u) << 23);
          const int shift = a < OZ_NACC - 1 ? u - 8 * a : 0;
          uint32_t v[N / 16][8];
#pragma unroll
          for (int x = 0; x < N / 16; x++)
            tmem_ld8(lane_addr + p * N + cbase + 8 * x, v[x]);
          tmem_ld_wait();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&slot_empty[p]);
#pragma unroll
          for (int x = 0; x < N / 16; x++)
#pragma unroll
            for (int y = 0; y < 8; y++)
              S[8 * x + y] += (long long)oz_to_int(__uint_as_float(v[x][y]), scale) << shift;
          sm.retire(a);
          if (!done) sch.advance(a);
        }
      }
      if (abort_flag) break;
      // C = S * 2^(e_r + f_c - 16 - u)
      double *C = (double *)J.g.C + T.c_off;
      const int64_t rowB = T.ecol;
      const int32_t *expB = J.expB;
      if (J.cls) {
        // class layout: the tile's rows and columns belong to several output
        // blocks; each element goes to (its row's A free box, its column's B
        // free box) at (row within the box) + (column within the box) * rows
        if (row_ok) {
          const OzRowMap ra_ = J.rmapA[T.erow + grow];
#pragma unroll
          for (int y0 = 0; y0 < N / 2; y0 += 8) {
            int fc[8];
            int64_t dst[8];
#pragma unroll
            for (int y = 0; y < 8; y++) {
              const int64_t gcol = T.nt * N + cbase + y0 + y;
              fc[y] = 0;
              dst[y] = -1;
              if (gcol < T.n) {
                fc[y] = __ldg(expB + rowB + gcol);
                const OzRowMap cb = J.rmapB[rowB + gcol];
                dst[y] = __ldg(J.offs + ra_.xoff + cb.xi) + ra_.xr + (int64_t)cb.xr * ra_.m;
              }
            }
#pragma unroll
            for (int y = 0; y < 8; y++)
              if (dst[y] >= 0) C[dst[y]] = oz_i64_ldexp(S[y0 + y], er + fc[y] - 16 - u);
          }
        }
      } else if (row_ok) {
        // the column exponents of 8 columns are loaded before their stores, so
        // the loads are not held behind stores that might alias them
#pragma unroll
        for (int y0 = 0; y0 < N / 2; y0 += 8) {
          int fc[8];
#pragma unroll
          for (int y = 0; y < 8; y++) {
            const int64_t gcol = T.nt * N + cbase + y0 + y;
            fc[y] = gcol < T.n ? __ldg(expB + rowB + gcol) : 0;
          }
#pragma unroll
          for (int y = 0; y < 8; y++) {
            const int64_t gcol = T.nt * N + cbase + y0 + y;
            if (gcol < T.n) C[grow + gcol * T.m] = oz_i64_ldexp(S[y0 + y], er + fc[y] - 16 - u);
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
int oz_stages(int s, int tile_n) {
  const int stage = s * ((OZ_M + tile_n) / 8) * 256;
  int n = OZ_SMEM_BYTES / stage;
  return n > OZ_MAX_STAGES ? OZ_MAX_STAGES : n;
}

static tq_status oz_setup(int *sms);

tq_status oz_batch_build(const std::vector<OzJob> &jobs, const std::vector<OzSide> &sides,
                         cudaStream_t st, OzBatchDev &out) {
  TQ_CHECK(oz_setup(&out.sms));
  const int64_t nj = (int64_t)jobs.size(), ns = (int64_t)sides.size();
  std::vector<int64_t> pre((nj + 1) + 3 * (ns + 1), 0);
  int64_t *jt = pre.data(), *sr = jt + nj + 1, *stl = sr + ns + 1, *se = stl + ns + 1;
  int s_max = 1;
  const int tile_n = nj ? jobs[0].tile_n : OZ_N;
  for (int64_t j = 0; j < nj; j++) {
    jt[j + 1] = jt[j] + jobs[j].n_tiles;
    s_max = jobs[j].s > s_max ? jobs[j].s : s_max;
    if (jobs[j].tile_n != tile_n)
      return fail(TQ_ERR_INVALID, "the jobs of one tensor-core launch must share the tile width");
  }
  if (tile_n != 32 && tile_n != 64 && tile_n != 96)
    return fail(TQ_ERR_INVALID, "tile width must be 32, 64 or 96");
  for (int64_t k = 0; k < ns; k++) {
    sr[k + 1] = sr[k] + sides[k].n_rows;
    stl[k + 1] = stl[k] + sides[k].n_tiles;
    se[k + 1] = se[k] + sides[k].n_exps;
  }
  TQ_CHECK(out.jobs.alloc(std::max<int64_t>(nj, 1), st));
  TQ_CHECK(out.sides.alloc(std::max<int64_t>(ns, 1), st));
  TQ_CHECK(out.prefixes.alloc(pre.size(), st));
  TQ_CHECK(out.err.alloc(1, st));
  if (nj) TQ_CUDA(cudaMemcpyAsync(out.jobs.p, jobs.data(), nj * sizeof(OzJob),
                                  cudaMemcpyHostToDevice, st));
  if (ns) TQ_CUDA(cudaMemcpyAsync(out.sides.p, sides.data(), ns * sizeof(OzSide),
                                  cudaMemcpyHostToDevice, st));
  TQ_CUDA(cudaMemcpyAsync(out.prefixes.p, pre.data(), pre.size() * 8, cudaMemcpyHostToDevice, st));
  TQ_CUDA(cudaMemsetAsync(out.err.p, 0, 4, st));
  TQ_CUDA(cudaStreamSynchronize(st));  // the host vectors die here
  OzLaunch &L = out.L;
  L.jobs = out.jobs.p;
  L.job_tile_start = out.prefixes.p;
  L.n_jobs = (int32_t)nj;
  L.n_tiles = jt[nj];
  L.sides = out.sides.p;
  L.side_row_start = out.prefixes.p + (nj + 1);
  L.side_tile_start = L.side_row_start + (ns + 1);
  L.side_exp_start = L.side_tile_start + (ns + 1);
  L.n_sides = (int32_t)ns;
  L.n_rows = sr[ns];
  L.n_slice_tiles = stl[ns];
  L.n_exps = se[ns];
  L.s_max = s_max;
  L.tile_n = tile_n;
  L.nstages = oz_stages(s_max, tile_n);
  L.err = out.err.p;
  TQ_CHECK(out.tiles.alloc(std::max<int64_t>(L.n_tiles, 1), st));
  L.tiles = out.tiles.p;
  if (L.n_tiles) {
    const unsigned g = (unsigned)((L.n_tiles + 255) / 256);
    count_launch();
    switch (tile_n) {
      case 32: oz_table_kernel<32><<<g, 256, 0, st>>>(L, out.tiles.p); break;
      case 64: oz_table_kernel<64><<<g, 256, 0, st>>>(L, out.tiles.p); break;
      default: oz_table_kernel<96><<<g, 256, 0, st>>>(L, out.tiles.p); break;
    }
    TQ_CUDA(cudaGetLastError());
  }
  return TQ_OK;
}

tq_status oz_batch_prepare(const OzBatchDev &b, cudaStream_t st) {
  const OzLaunch &L = b.L;
  const int T = 256;
  if (L.n_exps) count_launch(), oz_exp_init_kernel<<<(unsigned)((L.n_exps + T - 1) / T), T, 0, st>>>(L);
  if (L.n_rows) count_launch(), oz_rowexp_kernel<<<(unsigned)((L.n_rows + T - 1) / T), T, 0, st>>>(L);
  if (L.n_slice_tiles) count_launch(), oz_slice_kernel<<<(unsigned)L.n_slice_tiles, 256, 0, st>>>(L);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

// Device attributes and the kernel's shared-memory opt-in, once per device and
// before any stream capture (called when a batch is built).
static int g_sms[128] = {0};

static tq_status oz_setup(int *sms) {
  int dev = 0;
  TQ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(TQ_ERR_UNSUPPORTED, "device ordinal above 127");
  if (!g_sms[dev]) {
    int n = 0;
    TQ_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    TQ_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 OZ_SMEM_BYTES));
    TQ_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 OZ_SMEM_BYTES));
    TQ_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<96>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 OZ_SMEM_BYTES));
    g_sms[dev] = n;
  }
  *sms = g_sms[dev];
  return TQ_OK;
}

tq_status oz_batch_gemm(const OzBatchDev &b, cudaStream_t st) {
  const OzLaunch &L = b.L;
  if (L.n_tiles == 0) return TQ_OK;
  const int64_t grid = L.n_tiles < b.sms ? L.n_tiles : b.sms;
  count_launch();
  switch (L.tile_n) {
    case 32: oz_gemm_kernel<32><<<(unsigned)grid, OZ_THREADS, OZ_SMEM_BYTES, st>>>(L); break;
    case 64: oz_gemm_kernel<64><<<(unsigned)grid, OZ_THREADS, OZ_SMEM_BYTES, st>>>(L); break;
    default: oz_gemm_kernel<96><<<(unsigned)grid, OZ_THREADS, OZ_SMEM_BYTES, st>>>(L); break;
  }
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

tq_status oz_batch_check(const OzBatchDev &b, cudaStream_t st) {
  int32_t e = 0;
  TQ_CUDA(cudaMemcpyAsync(&e, b.err.p, 4, cudaMemcpyDeviceToHost, st));
  TQ_CUDA(cudaStreamSynchronize(st));
  if (e) {
    TQ_CUDA(cudaMemsetAsync(b.err.p, 0, 4, st));
    return fail(TQ_ERR_TIMEOUT,
                "a tensor-core pipeline wait gave up (flags " + std::to_string(e) + ")");
  }
  return TQ_OK;
}

}  // namespace tq
