// The persistent tensor-core GEMM of the sliced forms (its method and operand
// layout are described at the top of gemm_ozaki.cu).  The kernel template is
// instantiated per tile width and slice specialisation in the gemm_ozaki_s*.cu
// translation units, which compile in parallel.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "gemm.cuh"
#include "ozaki.cuh"
#include "sm100_ptx.cuh"

namespace tq {

constexpr int OZ_THREADS = 320;  // warp 0: loads, warp 1: MMA, warps 2-9: epilogue
constexpr uint32_t OZ_TMEM_COLS = 512;
// TMEM: OZ_NACC + 1 slots of tile-width columns (at most 480 of 512)
constexpr int OZ_NACC = 4;
constexpr int OZ_SMEM_BYTES = 216 * 1024;  // three two-k-step stages of five slices

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
  // (at most 2: a copy into tensor memory costs the tensor pipe about as much
  // as an MMA, and pays only for the slices that several products read)
  static constexpr int ntm = ((int)OZ_TMEM_COLS - n * N) / 8 < 2 ? ((int)OZ_TMEM_COLS - n * N) / 8 : 2;
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

// Binary16 operands: the OZ_F16_PACK k-steps of a packed step, each one MMA
// (A and B from shared memory) into the one accumulator.
__device__ __forceinline__ void oz_issue_packed(uint32_t col0, uint64_t da0, uint64_t db0,
                                                uint32_t a_step, uint32_t b_step, uint32_t idesc,
                                                uint32_t fresh) {
#pragma unroll
  for (int t = 0; t < OZ_F16_PACK; t++)
    mma_bf16(col0, da0 + (uint64_t)(t * a_step), db0 + (uint64_t)(t * b_step), idesc,
             (t == 0 && (fresh & 1)) ? 0u : 1u);
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
  int64_t chunk;
  // ks (packed) steps; accumulators retire every `pack`-th of OZ_CHUNK steps
  __device__ __forceinline__ void start(int64_t ks, int na, int pack = 1) {
    ksum = ks;
    n_acc = na;
    chunk = OZ_CHUNK / pack;
    const int stag = OZ_STAG / pack;
#pragma unroll
    for (int a = 0; a < OZ_NACC; a++) next[a] = chunk - stag * a;
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
    if (kind != OZ_FINAL) next[kind] += chunk;
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

// S > 0: every job of the launch has S slices (straight-line issue code);
// S = 0: any slice count (dispatched per job); S = OZ_F16: binary16 operands
// taken as they are (one "slice", kind::f16 with fp16 A and B, fp32
// accumulation in TMEM, retired accumulators summed in fp32, one rounding of
// each result element to binary16).
constexpr int OZ_F16 = -1;

template <int N, int S>
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
      // failure-path test hook: the producer holds back before it arms any
      // barrier or issues any copy, so the other roles' bounded waits run out
      // (then it sees the abort flag and issues nothing)
      if (L.delay_ns) {
        const uint64_t t0 = global_ns();
        while (global_ns() - t0 < L.delay_ns) __nanosleep(1000);
      }
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
        const int pack = S == OZ_F16 ? 1 : S > 0 ? oz_pack_for(S) : J.pack;
        const int se = s * pack;  // slices of a stored step
        const OzPairRec *prs = J.prs;
        const uint8_t *sliceA = J.sliceA, *sliceB = J.sliceB;
        const uint32_t ba = (uint32_t)se * T.ga * 256, bb = (uint32_t)se * T.gb * 256;
        const int n_acc = S == OZ_F16 ? 1 : s < OZ_NACC ? s : OZ_NACC;
        OzSchedule sch;
        sch.start(T.ksum, n_acc, pack);
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
          const uint8_t *ga = sliceA + pr.a_off + nk * se * 256 * (OZ_M / 8) * T.mt;
          const uint8_t *gb = sliceB + pr.b_off + nk * se * 256 * (N / 8) * T.nt;
          for (int64_t q = 0; q < nk; q++, it++) {
            if (it >= (uint32_t)NS && !mbar_wait(&empty_bar[st], ph, L.wait_ns)) {
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
                    !mbar_wait(&slot_empty[p], sm.drain_parity(p), L.wait_ns))
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
        if (!mbar_wait(&full_bar[q % NS], (q / NS) & 1, L.wait_ns)) atomicOr(L.err, 2);
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
        const int pack = S == OZ_F16 ? 1 : S > 0 ? oz_pack_for(S) : J.pack;
        const int n_acc = S == OZ_F16 ? 1 : s < OZ_NACC ? s : OZ_NACC;
        const OzPairRec *prs = J.prs;
        const uint32_t idesc = S == OZ_F16 ? idesc_f16_f32(OZ_M, (uint32_t)T.nmma)
                                           : idesc_bf16_f32(OZ_M, (uint32_t)T.nmma);
        OzSchedule sch;
        sch.start(T.ksum, n_acc, pack);
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
            if (lane == 0) ok = mbar_wait(&full_bar[st], ph, L.wait_ns);
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
              // the stage's k-steps one after another: k-step j's slices follow
              // k-step j-1's; accumulators restart only with the first
              const uint32_t as = (uint32_t)T.ga * 16, bs = (uint32_t)T.gb * 16;
              if constexpr (S == OZ_F16) {
                oz_issue_packed(col[0], dA0 + so, dB0 + so, as, bs, idesc, fresh);
              } else if constexpr (S > 0) {
                constexpr int PK = oz_pack_for(S);
#pragma unroll
                for (int j = 0; j < PK; j++)
                  oz_issue<S, true, OzSlots<N>::ntm>(
                      col, dA0 + so + (uint64_t)(j * S) * as, dB0 + so + (uint64_t)(j * S) * bs,
                      as, bs, idesc, j == 0 ? fresh : 0u, tmem + NSLOT * N);
              } else {
                for (int j = 0; j < pack; j++)
                  oz_issue_s<true, OzSlots<N>::ntm>(
                      s, col, dA0 + so + (uint64_t)(j * s) * as, dB0 + so + (uint64_t)(j * s) * bs,
                      as, bs, idesc, j == 0 ? fresh : 0u, tmem + NSLOT * N);
              }
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
      if (lane == 0 && !mbar_wait(&done_bar, 0, L.wait_ns)) atomicOr(L.err, 32);
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
      const int n_acc = S == OZ_F16 ? 1 : J.s < OZ_NACC ? J.s : OZ_NACC;
      const int pack = S == OZ_F16 ? 1 : S > 0 ? oz_pack_for(S) : J.pack;
      const int64_t grow = T.mt * OZ_M + row;
      const bool row_ok = grow < T.m;
      const int er = S != OZ_F16 && row_ok ? J.expA[T.erow + grow] : 0;
      // S: running sum in units of 2^-u of the leading slice product.  With
      // u <= 48 - log2(K) the sum stays below 2^62.1 for any data, and u >= 24
      // keeps D0..D2 (whole multiples of 2^-16) exact.
      int kb = 0;
      while (kb < 40 && (int64_t(1) << kb) < 16 * pack * T.ksum) kb++;
      const int u = 48 - kb < 32 ? 48 - kb : 32;
      // binary16 operands: a plain fp32 sum of the retired fp32 accumulators
      // (FP64 adds here would outlast the MMAs: GB300's FP64 rate is ~1/60 of
      // fp32; 2^-24 per fold is far below the result's binary16 rounding)
      std::conditional_t<S == OZ_F16, float, long long> sum[N / 2];
#pragma unroll
      for (int y = 0; y < N / 2; y++) sum[y] = 0;
      OzSchedule sch;
      sch.start(T.ksum, n_acc, pack);
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
          if (!mbar_wait(&slot_full[p], ((sm.par >> p) & 1), L.wait_ns)) {
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
            for (int y = 0; y < 8; y++) {
              if constexpr (S == OZ_F16)
                sum[8 * x + y] += __uint_as_float(v[x][y]);
              else
                sum[8 * x + y] += (long long)oz_to_int(__uint_as_float(v[x][y]), scale) << shift;
            }
          sm.retire(a);
          if (!done) sch.advance(a);
        }
      }
      if (abort_flag) break;
      if constexpr (S == OZ_F16) {
        // binary16 result: each element rounded once from the fp32 sum
        __half *C = (__half *)J.g.C + T.c_off;
        if (J.cls) {
          if (row_ok) {
            const OzRowMap ra_ = J.rmapA[T.erow + grow];
#pragma unroll
            for (int y = 0; y < N / 2; y++) {
              const int64_t gcol = T.nt * N + cbase + y;
              if (gcol < T.n) {
                const OzRowMap cb = J.rmapB[T.ecol + gcol];
                C[__ldg(J.offs + ra_.xoff + cb.xi) + ra_.xr + (int64_t)cb.xr * ra_.m] =
                    __float2half_rn(sum[y]);
              }
            }
          }
        } else if (row_ok) {
#pragma unroll
          for (int y = 0; y < N / 2; y++) {
            const int64_t gcol = T.nt * N + cbase + y;
            if (gcol < T.n) C[grow + gcol * T.m] = __float2half_rn(sum[y]);
          }
        }
        continue;
      }
      // C = sum * 2^(e_r + f_c - 16 - u)
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
              if (dst[y] >= 0) C[dst[y]] = oz_i64_ldexp(sum[y0 + y], er + fc[y] - 16 - u);
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
            if (gcol < T.n) C[grow + gcol * T.m] = oz_i64_ldexp(sum[y0 + y], er + fc[y] - 16 - u);
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

// Shared-memory opt-in of the three tile widths of slice specialisation S.
template <int S>
tq_status oz_gemm_set_attr() {
  TQ_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<32, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               OZ_SMEM_BYTES));
  TQ_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<64, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               OZ_SMEM_BYTES));
  TQ_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<96, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               OZ_SMEM_BYTES));
  return TQ_OK;
}

template <int S>
tq_status oz_gemm_run(const OzLaunch &L, unsigned grid, cudaStream_t st) {
  switch (L.tile_n) {
    case 32: oz_gemm_kernel<32, S><<<grid, OZ_THREADS, OZ_SMEM_BYTES, st>>>(L); break;
    case 64: oz_gemm_kernel<64, S><<<grid, OZ_THREADS, OZ_SMEM_BYTES, st>>>(L); break;
    default: oz_gemm_kernel<96, S><<<grid, OZ_THREADS, OZ_SMEM_BYTES, st>>>(L); break;
  }
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

// The instantiations: S = 0 (any slice count), 3 (three-way bf16), 5 (the
// FP64-level default) and OZ_F16 (binary16 operands), one translation unit each.
tq_status oz_gemm_set_attr_s0();
tq_status oz_gemm_set_attr_s3();
tq_status oz_gemm_set_attr_s5();
tq_status oz_gemm_run_s0(const OzLaunch &L, unsigned grid, cudaStream_t st);
tq_status oz_gemm_run_s3(const OzLaunch &L, unsigned grid, cudaStream_t st);
tq_status oz_gemm_run_s5(const OzLaunch &L, unsigned grid, cudaStream_t st);
tq_status oz_gemm_set_attr_f16();
tq_status oz_gemm_run_f16(const OzLaunch &L, unsigned grid, cudaStream_t st);

}  // namespace tq
