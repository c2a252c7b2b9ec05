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
#include <cuda_fp16.h>

#include <atomic>

#include "gemm.cuh"
#include "oz_gemm.cuh"
#include "ozaki.cuh"
#include "sm100_ptx.cuh"

namespace tq {


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
  if (S.f16) return;  // binary16 operands are not scaled
  const int64_t lr = g - L.side_row_start[k];
  const int64_t b = oz_find(S.row_start, S.T.nb, lr);
  const int64_t r = lr - S.row_start[b];
  Operand op;
  side_operand(S, b, op);
  const double *d = (const double *)S.T.data;
  const int64_t ra = op.base + mixed_addr(r, op.nr, op.rdim, op.rst);
  // eight independent loads in flight per iteration (the loop is bound by
  // load latency, not by arithmetic)
  unsigned long long m8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int64_t c = 0;
  for (; c + 8 <= op.cols; c += 8) {
#pragma unroll
    for (int x = 0; x < 8; x++) {
      const unsigned long long bits = (unsigned long long)__double_as_longlong(
                                          d[ra + mixed_addr(c + x, op.nc, op.cdim, op.cst)]) &
                                      0x7fffffffffffffffull;
      m8[x] = bits > m8[x] ? bits : m8[x];
    }
  }
  for (; c < op.cols; c++) {
    const unsigned long long bits =
        (unsigned long long)__double_as_longlong(d[ra + mixed_addr(c, op.nc, op.cdim, op.cst)]) &
        0x7fffffffffffffffull;
    m8[0] = bits > m8[0] ? bits : m8[0];
  }
  unsigned long long mx = 0;
#pragma unroll
  for (int x = 0; x < 8; x++) mx = m8[x] > mx ? m8[x] : mx;
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

// The 8 values of half row c (columns q*16 + c*8 ..) of row r (absent ones 0).
__device__ __forceinline__ void oz_load8(const double *d, bool row_ok, int64_t ra,
                                         const Operand &op, int64_t q, int c, double (&v)[8]) {
#pragma unroll
  for (int x = 0; x < 8; x++) {
    const int64_t kk = q * 16 + c * 8 + x;
    v[x] = row_ok && kk < op.cols ? d[ra + mixed_addr(kk, op.nc, op.cdim, op.cst)] : 0.0;
  }
}

// The s slices of one half row (its 8 values v) of row r of an operand row
// tile with G row groups, written into the k-step's chunk.
__device__ __forceinline__ void oz_slice_kstep(const double (&v)[8], int c, int shift, int s, int G,
                                               int r, uint8_t *chunk) {
  uint32_t packed[OZ_MAXS][4];
#pragma unroll
  for (int t = 0; t < OZ_MAXS; t++)
#pragma unroll
    for (int w = 0; w < 4; w++) packed[t][w] = 0;
#pragma unroll
  for (int x = 0; x < 8; x++) {
    long long F = oz_fixed(v[x], shift);
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

// All nk k-steps of one half row: the loads of k-step q+1 are issued before
// k-step q is split and stored, so each thread keeps loads in flight.
__device__ __forceinline__ void oz_slice_rows(const double *d, bool row_ok, int64_t ra,
                                              const Operand &op, int64_t nk, int c, int shift,
                                              int s, int G, int r, uint8_t *base) {
  if (nk <= 0) return;
  double cur[8], nxt[8];
  oz_load8(d, row_ok, ra, op, 0, c, cur);
  for (int64_t q = 0; q < nk; q++) {
    if (q + 1 < nk) oz_load8(d, row_ok, ra, op, q + 1, c, nxt);
    oz_slice_kstep(cur, c, shift, s, G, r, base + q * (int64_t)s * G * 256);
#pragma unroll
    for (int x = 0; x < 8; x++) cur[x] = nxt[x];
  }
}

// Binary16 operands as they are: the 8 half values of half row c of row r in
// k-step q, in the same core-matrix image (one slice).
__device__ __forceinline__ void oz_copy_kstep_f16(const __half *d, bool row_ok, int64_t ra,
                                                  const Operand &op, int64_t q, int c, int G,
                                                  int r, uint8_t *chunk) {
  uint32_t packed[4] = {0, 0, 0, 0};
#pragma unroll
  for (int x = 0; x < 8; x++) {
    const int64_t kk = q * 16 + c * 8 + x;
    uint32_t h = 0;
    if (row_ok && kk < op.cols) h = __half_as_ushort(d[ra + mixed_addr(kk, op.nc, op.cdim, op.cst)]);
    packed[x >> 1] |= h << (16 * (x & 1));
  }
  *(uint4 *)(chunk + ((r / 8) * 2 + c) * 128 + (r % 8) * 16) =
      make_uint4(packed[0], packed[1], packed[2], packed[3]);
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
  // it.koff and it.nk count stored steps of S.pack k-steps
  uint8_t *base = S.slices + 256 * it.unit + (int64_t)it.koff * S.pack * s * G * 256;
  if (S.f16) {
    // it.nk packed steps of OZ_F16_PACK k-steps; the padding k-steps are zeros
    for (int64_t q = 0; q < it.nk * OZ_F16_PACK; q++)
      oz_copy_kstep_f16((const __half *)S.T.data, row_ok, ra, op, q, c, G, r,
                        base + q * (int64_t)G * 256);
    return;
  }
  oz_slice_rows((const double *)S.T.data, row_ok, ra, op, (int64_t)it.nk * S.pack, c, 8 * s - e, s,
                G, r, base);
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
  const int64_t kw = oz_kstep_cols(S.f16, S.pack);
  const int64_t nk = (op.cols + kw - 1) / kw * S.pack;  // 16-column k-steps (zero past cols)
  uint8_t *base = S.slices + 256 * S.unit_off[b] + nk * (int64_t)s * 256 * (rt_rows / 8) * rt;
  const int r = threadIdx.x >> 1, c = threadIdx.x & 1;
  if (r >= G * 8) return;
  const int64_t grow = rt * rt_rows + r;
  const bool row_ok = r < rows;
  const int64_t ra = row_ok ? op.base + mixed_addr(grow, op.nr, op.rdim, op.rst) : 0;
  if (S.f16) {
    for (int64_t q = 0; q < nk * OZ_F16_PACK; q++)
      oz_copy_kstep_f16((const __half *)S.T.data, row_ok, ra, op, q, c, G, r,
                        base + q * (int64_t)G * 256);
    return;
  }
  const int e = row_ok ? S.exps[S.row_off[S.key[b]] + grow] : OZ_EXP_ZERO;
  oz_slice_rows((const double *)S.T.data, row_ok, ra, op, nk, c, 8 * s - e, s, G, r, base);
}

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

// ---------------------------------------------------------------- host side
int oz_stages(int s, int tile_n) {
  const int stage = s * ((OZ_M + tile_n) / 8) * 256;
  int n = OZ_SMEM_BYTES / stage;
  return n > OZ_MAX_STAGES ? OZ_MAX_STAGES : n;
}

static tq_status oz_setup(int *sms);

// Pipeline wait limit and producer delay of the launches built from now on
// (tq_debug_set_waits; the defaults are 2 s and none).
static std::atomic<uint64_t> g_wait_ns{2000000000ull}, g_delay_ns{0};
static void debug_waits(uint64_t *wait_ns, uint64_t *delay_ns) {
  *wait_ns = g_wait_ns.load();
  *delay_ns = g_delay_ns.load();
}

tq_status oz_batch_build(const std::vector<OzJob> &jobs, const std::vector<OzSide> &sides,
                         cudaStream_t st, OzBatchDev &out) {
  TQ_CHECK(oz_setup(&out.sms));
  const int64_t nj = (int64_t)jobs.size(), ns = (int64_t)sides.size();
  std::vector<int64_t> pre((nj + 1) + 3 * (ns + 1), 0);
  int64_t *jt = pre.data(), *sr = jt + nj + 1, *stl = sr + ns + 1, *se = stl + ns + 1;
  int s_max = 1;
  const int tile_n = nj ? jobs[0].tile_n : OZ_N;
  const int32_t f16 = nj ? jobs[0].f16 : 0;
  for (int64_t j = 0; j < nj; j++) {
    if (jobs[j].f16 != f16)
      return fail(TQ_ERR_UNSUPPORTED, "binary16 and float64 jobs cannot share a tensor-core launch");
    jt[j + 1] = jt[j] + jobs[j].n_tiles;
    // a stage holds one stored step: s slices of `pack` k-steps
    const int se_j = jobs[j].s * (jobs[j].pack > 0 ? jobs[j].pack : 1);
    s_max = se_j > s_max ? se_j : s_max;
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
  L.s_all = nj ? jobs[0].s : 0;
  for (int64_t j = 0; j < nj; j++)
    if (jobs[j].s != L.s_all || jobs[j].pack != oz_pack_of(jobs[j].s, jobs[j].f16)) L.s_all = 0;
  L.tile_n = tile_n;
  L.f16 = f16;
  L.nstages = oz_stages(s_max, tile_n);
  L.err = out.err.p;
  debug_waits(&L.wait_ns, &L.delay_ns);
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
    TQ_CHECK(oz_gemm_set_attr_s0());
    TQ_CHECK(oz_gemm_set_attr_s3());
    TQ_CHECK(oz_gemm_set_attr_s5());
    TQ_CHECK(oz_gemm_set_attr_f16());
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
  if (L.f16) return oz_gemm_run_f16(L, (unsigned)grid, st);
  // straight-line issue code when every job of the launch has 3 or 5 slices
  if (L.s_all == 5) return oz_gemm_run_s5(L, (unsigned)grid, st);
  if (L.s_all == 3) return oz_gemm_run_s3(L, (unsigned)grid, st);
  return oz_gemm_run_s0(L, (unsigned)grid, st);
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

extern "C" void tq_debug_set_waits(uint64_t wait_ns, uint64_t producer_delay_ns) {
  tq::g_wait_ns.store(wait_ns ? wait_ns : 2000000000ull);
  tq::g_delay_ns.store(producer_delay_ns);
}
