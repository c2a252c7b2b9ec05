// contract: the symbolic stage (index kernels, output boxes and offsets) and
// the numeric stage (grouped GEMM) of torque::gpu::BlockSparseTensor::contract
// (src/gpu/block_sparse.cuh:558-1026).
//
// Symbolic stage, all on the device:
//   1. match: per A block the B blocks whose contracted intervals overlap
//      (counts -> exclusive scan -> ordered emit): the pair list in the
//      reference's order, A ascending then B ascending (block_sparse.cuh:626-652);
//   2. output boxes: A free legs ++ B free legs of each pair
//      (src/tensor/block_sparse.cpp:66-119); offsets = exclusive scan of the
//      element counts (block_sparse.cuh:658-674);
//   3. reduced layout only: pairs keyed by their output box (interval ids of the
//      free legs), stably radix-sorted, segmented: one output block per key.
// One host synchronisation reads the sizes and allocates the result.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "gemm.cuh"
#include "index.cuh"
#include "ozaki.cuh"
#include "plan.cuh"

namespace tq {

// ---------------------------------------------------------------- kernels
__global__ void pair_stats_kernel(DevBS A, DevBS B, LegSpec L, const int32_t *pa,
                                  const int32_t *pb, int64_t n_pairs, int64_t *mnk,
                                  int64_t *chunks) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const int64_t i = pa[p], j = pb[p];
  int64_t m = 1, n = 1, k = 1;
  for (int q = 0; q < L.nfa; q++)
    m *= A.end[i * A.rank + L.fa[q]] - A.begin[i * A.rank + L.fa[q]] + 1;
  for (int q = 0; q < L.nfb; q++)
    n *= B.end[j * B.rank + L.fb[q]] - B.begin[j * B.rank + L.fb[q]] + 1;
  int64_t cb[TQ_MAXR], ce[TQ_MAXR];
  contraction_range(A, B, L, i, j, cb, ce);
  for (int c = 0; c < L.nc; c++) k *= ce[c] - cb[c] + 1;
  mnk[p] = m * n * k;
  if (chunks) chunks[p] = (k + DOT_CHUNK - 1) / DOT_CHUNK;
}

// Output block o: box of its first pair; column-major strides; element and
// tile counts.
__global__ void out_meta_kernel(DevBS A, DevBS B, LegSpec L, const int32_t *pa,
                                const int32_t *pb, const int64_t *seg, const int64_t *perm,
                                int64_t n_out, int32_t rc, int64_t *c_begin, int64_t *c_end,
                                int64_t *c_strides, int64_t *n_elem, int64_t *tiles) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_out) return;
  const int64_t p0 = perm ? perm[seg[o]] : seg[o];
  const int64_t i = pa[p0], j = pb[p0];
  int64_t stride = 1, m = 1, n = 1;
  for (int q = 0; q < rc; q++) {
    int64_t b, e;
    if (q < L.nfa) {
      b = A.begin[i * A.rank + L.fa[q]];
      e = A.end[i * A.rank + L.fa[q]];
      m *= e - b + 1;
    } else {
      b = B.begin[j * B.rank + L.fb[q - L.nfa]];
      e = B.end[j * B.rank + L.fb[q - L.nfa]];
      n *= e - b + 1;
    }
    c_begin[o * rc + q] = b;
    c_end[o * rc + q] = e;
    c_strides[o * rc + q] = stride;
    stride *= e - b + 1;
  }
  n_elem[o] = stride;
  tiles[o] = ((m + NT_TM - 1) / NT_TM) * ((n + NT_TN - 1) / NT_TN);
}

__global__ void iota_kernel(int64_t *x, int64_t n) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) x[p] = p;
}

// --- interval ids of one leg (for the reduced layout) ------------------------
// For every block: its interval [b, e] on `leg`.  The leg is "laminar" when any
// two intervals are equal or disjoint; the id of an interval is then the rank
// of its begin among all begins.
__global__ void mark_intervals_kernel(DevBS T, int32_t leg, int64_t *is_begin,
                                      unsigned long long *emin, unsigned long long *emax) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= T.nb) return;
  const int64_t x = T.begin[b * T.rank + leg];
  const unsigned long long e = (unsigned long long)T.end[b * T.rank + leg];
  is_begin[x] = 1;
  atomicMin(&emin[x], e);
  atomicMax(&emax[x], e);
}

__global__ void check_intervals_kernel(const int64_t *is_begin, const int64_t *ids, int64_t dim,
                                       const unsigned long long *emin,
                                       const unsigned long long *emax, int64_t *begin_of_id,
                                       int32_t *bad) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= dim || !is_begin[x]) return;
  if (emin[x] != emax[x]) atomicOr(bad, 1);
  begin_of_id[ids[x]] = x;
}

// n_ids is read on the device (the scan's total); the grid covers the leg's
// dimension, an upper bound of it.
__global__ void check_disjoint_kernel(const int64_t *begin_of_id, const int64_t *n_ids,
                                      const unsigned long long *emax, int32_t *bad) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t + 1 >= *n_ids) return;
  if ((int64_t)emax[begin_of_id[t]] >= begin_of_id[t + 1]) atomicOr(bad, 1);
}

// state[0] is the running mixed radix (the product of the earlier legs' id counts).
__global__ void block_key_kernel(DevBS T, int32_t leg, const int64_t *ids, const int64_t *state,
                                 int64_t *key) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= T.nb) return;
  key[b] += ids[T.begin[b * T.rank + leg]] * state[0];
}

// After a leg's keys: radix *= max(n_ids, 1), flagging (bad |= 2) a key range
// beyond 2^62.
__global__ void radix_step_kernel(const int64_t *n_ids, int64_t *state, int32_t *bad) {
  const int64_t n = *n_ids > 0 ? *n_ids : 1;
  if (state[0] > (int64_t(1) << 62) / n) {
    atomicOr(bad, 2);
    return;
  }
  state[0] *= n;
}

__global__ void box_keys_init_kernel(int64_t *state, int32_t *bad) {
  state[0] = 1;
  state[1] = 0;
  *bad = 0;
}

__global__ void box_keys_done_kernel(int64_t *state, const int32_t *bad) { state[1] = *bad; }

__global__ void pair_key_kernel(const int32_t *pa, const int32_t *pb, int64_t n,
                                const int64_t *ka, const int64_t *kb, int64_t KA, int64_t *key) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) key[p] = ka[pa[p]] + KA * kb[pb[p]];
}

__global__ void seg_flag_kernel(const int64_t *key, int64_t n, int64_t *flag) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) flag[s] = (s == 0 || key[s] != key[s - 1]) ? 1 : 0;
}

__global__ void seg_start_kernel(const int64_t *flag, const int64_t *sid, int64_t n,
                                 int64_t n_out, int64_t *seg) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n && flag[s]) seg[sid[s]] = s;
  if (s == 0) seg[n_out] = n;
}

static inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Interval-id keys of every block of T over `legs` (mixed radix, first leg
// fastest).  *K receives the key range; returns UNSUPPORTED if a leg is not
// laminar or the key range overflows.  The radix and the failure flags stay on
// the device across the legs: one host synchronisation per call.
static tq_status box_keys(const tq_bs *T, int32_t nlegs, const int32_t *legs, int64_t *key,
                          int64_t *K, cudaStream_t s) {
  TQ_CUDA(cudaMemsetAsync(key, 0, sizeof(int64_t) * std::max<int64_t>(T->nb, 1), s));
  *K = 1;
  if (nlegs == 0) return TQ_OK;
  DevArray<int32_t> bad;
  DevArray<int64_t> state;  // [radix, flags]
  TQ_CHECK(bad.alloc(1, s));
  TQ_CHECK(state.alloc(2, s));
  count_launch(), box_keys_init_kernel<<<1, 1, 0, s>>>(state.p, bad.p);
  const DevBS v = T->view();
  for (int32_t q = 0; q < nlegs; q++) {
    const int32_t leg = legs[q];
    const int64_t dim = T->dimension[leg];
    DevArray<int64_t> is_begin, ids, begin_of_id, total;
    DevArray<unsigned long long> emin, emax;
    TQ_CHECK(is_begin.alloc(dim, s));
    TQ_CHECK(ids.alloc(dim, s));
    TQ_CHECK(begin_of_id.alloc(dim, s));
    TQ_CHECK(total.alloc(1, s));
    TQ_CHECK(emin.alloc(dim, s));
    TQ_CHECK(emax.alloc(dim, s));
    TQ_CUDA(cudaMemsetAsync(is_begin.p, 0, dim * 8, s));
    TQ_CUDA(cudaMemsetAsync(emin.p, 0xff, dim * 8, s));
    TQ_CUDA(cudaMemsetAsync(emax.p, 0, dim * 8, s));
    count_launch(), mark_intervals_kernel<<<nblk(T->nb), 256, 0, s>>>(v, leg, is_begin.p, emin.p, emax.p);
    TQ_CHECK(scan_exclusive(is_begin.p, ids.p, dim, total.p, s));
    count_launch(), check_intervals_kernel<<<nblk(dim), 256, 0, s>>>(is_begin.p, ids.p, dim, emin.p, emax.p,
                                                     begin_of_id.p, bad.p);
    count_launch(), check_disjoint_kernel<<<nblk(std::max<int64_t>(dim, 1)), 256, 0, s>>>(
        begin_of_id.p, total.p, emax.p, bad.p);
    count_launch(), block_key_kernel<<<nblk(T->nb), 256, 0, s>>>(v, leg, ids.p, state.p, key);
    count_launch(), radix_step_kernel<<<1, 1, 0, s>>>(total.p, state.p, bad.p);
    TQ_CUDA(cudaGetLastError());
  }
  count_launch(), box_keys_done_kernel<<<1, 1, 0, s>>>(state.p, bad.p);
  TQ_CUDA(cudaGetLastError());
  int64_t h[2] = {1, 0};
  TQ_CUDA(cudaMemcpyAsync(h, state.p, 16, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  if (h[1] & 1)
    return fail(TQ_ERR_UNSUPPORTED,
                "reduced layout needs the free legs' intervals to be equal or disjoint "
                "(sector boxes); use the reference layout");
  if (h[1] & 2) return fail(TQ_ERR_UNSUPPORTED, "output box key range exceeds 2^62");
  *K = h[0];
  return TQ_OK;
}

static int bits_for(int64_t K) {
  int b = 0;
  while (b < 63 && (int64_t(1) << b) < K) b++;
  return b;
}

// ---------------------------------------------------------------- tensor-core plan
// The sliced forms take sector-aligned pairs: every matched pair covers the same
// full interval of both blocks on each contracted leg (true for charge-sector
// tensors), so each block is sliced once and shared by all its pairs.
__global__ void tc_align_kernel(DevBS A, DevBS B, LegSpec L, const int32_t *pa, const int32_t *pb,
                                int64_t n, int32_t *bad) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int64_t i = pa[p], j = pb[p];
  for (int k = 0; k < L.nc; k++)
    if (A.begin[i * A.rank + L.al[k]] != B.begin[j * B.rank + L.bl[k]] ||
        A.end[i * A.rank + L.al[k]] != B.end[j * B.rank + L.bl[k]])
      atomicOr(bad, 1);
}

__global__ void tc_block_stats_kernel(OzSide S, int32_t rt_rows, int32_t slices, int64_t *mkey,
                                      int64_t *rows, int64_t *tiles, int64_t *units) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= S.T.nb) return;
  int64_t m = 1, k = 1;
  for (int q = 0; q < S.nfree; q++)
    m *= S.T.end[b * S.T.rank + S.free_legs[q]] - S.T.begin[b * S.T.rank + S.free_legs[q]] + 1;
  for (int q = 0; q < S.ncon; q++)
    k *= S.T.end[b * S.T.rank + S.con[q]] - S.T.begin[b * S.T.rank + S.con[q]] + 1;
  rows[b] = m;
  tiles[b] = (m + rt_rows - 1) / rt_rows;
  const int64_t kw = oz_kstep_cols(S.f16, S.pack);
  units[b] = ((k + kw - 1) / kw) * S.pack * slices * ((m + 7) / 8);
  mkey[S.key[b]] = m;
}

// Per output block: k-steps of its pairs and its tensor-core tiles; with block
// grouping, outputs whose tiles would be filled to less than native_fill/1000
// get no tensor-core tiles and their native tiles (nt_native, the 64x64 tiling
// of the native kernel) instead.
__global__ void tc_out_kernel(DevBS A, DevBS B, LegSpec L, const int32_t *pa, const int32_t *pb,
                              const int64_t *seg, const int64_t *perm, int64_t n_out,
                              int32_t tile_n, int32_t native_fill, int32_t kw, int32_t *nk_pair,
                              int64_t *tiles, int64_t *ksum, int64_t *nt_native) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_out) return;
  int64_t tot = 0;
  for (int64_t sidx = seg[o]; sidx < seg[o + 1]; sidx++) {
    const int64_t p = perm ? perm[sidx] : sidx;
    const int64_t i = pa[p];
    int64_t k = 1;
    for (int q = 0; q < L.nc; q++)
      k *= A.end[i * A.rank + L.al[q]] - A.begin[i * A.rank + L.al[q]] + 1;
    nk_pair[p] = (int32_t)((k + kw - 1) / kw);
    tot += (k + kw - 1) / kw;
  }
  ksum[o] = tot;
  const int64_t p0 = perm ? perm[seg[o]] : seg[o];
  int64_t m = 1, n = 1;
  for (int q = 0; q < L.nfa; q++)
    m *= A.end[pa[p0] * A.rank + L.fa[q]] - A.begin[pa[p0] * A.rank + L.fa[q]] + 1;
  for (int q = 0; q < L.nfb; q++)
    n *= B.end[pb[p0] * B.rank + L.fb[q]] - B.begin[pb[p0] * B.rank + L.fb[q]] + 1;
  const int64_t t = ((m + OZ_M - 1) / OZ_M) * ((n + tile_n - 1) / tile_n);
  // fill = m n / (t OZ_M tile_n) < native_fill / 1000
  const bool native = m * n * 1000 < (int64_t)native_fill * t * OZ_M * tile_n;
  tiles[o] = native ? 0 : t;
  nt_native[o] = native ? ((m + NT_TM - 1) / NT_TM) * ((n + NT_TN - 1) / NT_TN) : 0;
}

// Split-K of the native kernel: per output its fused K, K chunks per tile
// (at most S, chunks of at least kmin columns), work items, reduced tiles and
// partial-tile slots.
__global__ void native_work_kernel(DevBS A, DevBS B, LegSpec L, const int32_t *pa,
                                   const int32_t *pb, const int64_t *seg, const int64_t *perm,
                                   int64_t n_out, const int64_t *tiles, int32_t S, int64_t kmin,
                                   int32_t *chunks, int64_t *kfused, int64_t *work,
                                   int64_t *nsplit, int64_t *slots) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_out) return;
  int64_t kf = 0;
  for (int64_t sidx = seg[o]; sidx < seg[o + 1]; sidx++) {
    const int64_t p = perm ? perm[sidx] : sidx;
    int64_t cb[TQ_MAXR], ce[TQ_MAXR], k = 1;
    contraction_range(A, B, L, pa[p], pb[p], cb, ce);
    for (int c = 0; c < L.nc; c++) k *= ce[c] - cb[c] + 1;
    kf += k;
  }
  int64_t ch = tiles[o] > 0 ? kf / kmin : 1;
  ch = ch < 1 ? 1 : (ch > S ? S : ch);
  chunks[o] = (int32_t)ch;
  kfused[o] = kf;
  work[o] = tiles[o] * ch;
  nsplit[o] = ch > 1 ? tiles[o] : 0;
  slots[o] = ch > 1 ? tiles[o] * ch : 0;
}

// The native launch over `total` tiles (tiles[o] per output, tile_start their
// exclusive scan): without split-K when the tiles alone give every SM about 8
// CTAs; otherwise each tile is cut into up to S K chunks.
static tq_status native_work(const tq_plan *P, const int64_t *tiles, const int64_t *tile_start,
                             int64_t total, NativeWorkDev &W, cudaStream_t s) {
  W.w = NativeWork{};
  W.w.n_work = total;
  W.w.work_start = tile_start;
  if (total == 0 || P->n_out == 0) return TQ_OK;
  int dev = 0, sms = 0;
  TQ_CUDA(cudaGetDevice(&dev));
  TQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t target = 8 * (int64_t)sms;
  if (total >= target) return TQ_OK;
  const int32_t S = (int32_t)std::min<int64_t>(32, (target + total - 1) / total);
  const int64_t no = P->n_out;
  DevArray<int64_t> work, nsplit, slots, tot;
  TQ_CHECK(W.chunks.alloc(no, s));
  TQ_CHECK(W.kfused.alloc(no, s));
  TQ_CHECK(W.work_start.alloc(no, s));
  TQ_CHECK(W.split_start.alloc(no, s));
  TQ_CHECK(W.split_off.alloc(no, s));
  TQ_CHECK(work.alloc(no, s));
  TQ_CHECK(nsplit.alloc(no, s));
  TQ_CHECK(slots.alloc(no, s));
  TQ_CHECK(tot.alloc(3, s));
  count_launch(), native_work_kernel<<<nblk(no), 256, 0, s>>>(
      P->A->view(), P->B->view(), P->L, P->pa.p, P->pb.p, P->seg.p, P->perm.p, no, tiles, S,
      (int64_t)256, W.chunks.p, W.kfused.p, work.p, nsplit.p, slots.p);
  TQ_CUDA(cudaGetLastError());
  TQ_CHECK(scan_exclusive(work.p, W.work_start.p, no, tot.p, s));
  TQ_CHECK(scan_exclusive(nsplit.p, W.split_start.p, no, tot.p + 1, s));
  TQ_CHECK(scan_exclusive(slots.p, W.split_off.p, no, tot.p + 2, s));
  int64_t h[3];
  TQ_CUDA(cudaMemcpyAsync(h, tot.p, 24, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  if (h[1] == 0) return TQ_OK;  // nothing long enough to split
  // partial tiles are held in the accumulation type (FP32 for binary16)
  const size_t acc_bytes = P->A->dtype == TQ_F64 ? 8 : 4;
  TQ_CHECK(W.scratch.alloc((size_t)h[2] * NT_TM * NT_TN * acc_bytes, s));
  W.w.n_work = h[0];
  W.w.n_split = h[1];
  W.w.work_start = W.work_start.p;
  W.w.split_start = W.split_start.p;
  W.w.split_off = W.split_off.p;
  W.w.chunks = W.chunks.p;
  W.w.kfused = W.kfused.p;
  W.w.scratch = W.scratch.p;
  return TQ_OK;
}

GemmJob make_gemm_job(const tq_plan *P) {
  GemmJob job;
  job.A = P->A->view();
  job.B = P->B->view();
  job.L = P->L;
  job.pa = P->pa.p;
  job.pb = P->pb.p;
  job.seg = P->seg.p;
  job.perm = P->perm.p;
  job.tile_start = P->tile_start.p;
  job.c_off = P->C->d_meta.p ? P->C->d_meta.p + 3 * P->n_out * P->C->rank : nullptr;
  job.C = P->out ? P->out : P->C->data;
  job.n_out = P->n_out;
  job.chunks = nullptr;
  job.kfused = nullptr;
  job.split_off = nullptr;
  job.scratch = nullptr;
  return job;
}

static OzSide make_side(const tq_bs *T, int32_t nfree, const int32_t *fl, int32_t ncon,
                        const int32_t *con, const int64_t *key, const int64_t *row_off,
                        const int64_t *row_start, const int64_t *tile_start,
                        const int64_t *unit_off) {
  OzSide S;
  std::memset(&S, 0, sizeof(S));
  S.T = T->view();
  S.nfree = nfree;
  S.ncon = ncon;
  for (int q = 0; q < nfree; q++) S.free_legs[q] = fl[q];
  for (int q = 0; q < ncon; q++) S.con[q] = con[q];
  S.key = key;
  S.row_off = row_off;
  S.row_start = row_start;
  S.tile_start = tile_start;
  S.unit_off = unit_off;
  S.f16 = T->dtype == TQ_F16;
  S.pack = 1;  // set with the slice count
  return S;
}

// ---------------------------------------------------------------- class layout
// The (A free box, B free box, pair count) of every output block.
__global__ void out_xy_kernel(const int32_t *pa, const int32_t *pb, const int64_t *seg,
                              const int64_t *perm, const int64_t *keyA, const int64_t *keyB,
                              int64_t n_out, int64_t *xy) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_out) return;
  const int64_t p0 = perm ? perm[seg[o]] : seg[o];
  xy[3 * o] = keyA[pa[p0]];
  xy[3 * o + 1] = keyB[pb[p0]];
  xy[3 * o + 2] = seg[o + 1] - seg[o];
}

template <typename T>
static tq_status upload(DevArray<T> &d, const std::vector<T> &h, cudaStream_t s) {
  TQ_CHECK(d.alloc(std::max<size_t>(h.size(), 1), s));
  if (!h.empty())
    TQ_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return TQ_OK;
}

// The class layout of the tensor-core forms (see OzClassOut), built when the
// contraction admits it: every free box's blocks carry distinct contracted boxes,
// and any two free boxes (one per side) that share a matched contracted box
// carry the same set of them.  Sets *used; leaves the plan as it was when the
// structure does not qualify (the per-block layout then runs).  Runs after the
// common part of plan_tc (row scans, exponent-table size); replaces the
// exponent-table offsets rowA / rowB by class order, so that the rows of a
// class are consecutive in the exponent tables and in its row map.
static tq_status plan_tc_classes(tq_plan *P, int32_t sl, int32_t tn, int64_t nexpA,
                                 int64_t nexpB, cudaStream_t s, bool *used) {
  *used = false;
  const tq_bs *A = P->A, *B = P->B;
  const LegSpec &L = P->L;
  const int64_t no = P->n_out;
  if (P->opts.layout != TQ_LAYOUT_REDUCED || P->opts.native_fill != 0 || no == 0 || L.nc == 0)
    return TQ_OK;
  TQ_CHECK(sync_host_meta(const_cast<tq_bs *>(A), s));
  TQ_CHECK(sync_host_meta(const_cast<tq_bs *>(B), s));
  TQ_CHECK(sync_host_meta(P->C, s));
  const int64_t na = A->nb, nbk = B->nb, KA = P->KA, KB = P->KB;
  std::vector<int64_t> keyA(na), keyB(nbk), xy(3 * no);
  {
    DevArray<int64_t> dxy;
    TQ_CHECK(dxy.alloc(3 * no, s));
    count_launch(), out_xy_kernel<<<nblk(no), 256, 0, s>>>(P->pa.p, P->pb.p, P->seg.p, P->perm.p,
                                                           P->keyA.p, P->keyB.p, no, dxy.p);
    TQ_CUDA(cudaGetLastError());
    TQ_CUDA(cudaMemcpyAsync(keyA.data(), P->keyA.p, na * 8, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaMemcpyAsync(keyB.data(), P->keyB.p, nbk * 8, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaMemcpyAsync(xy.data(), dxy.p, 3 * no * 8, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaStreamSynchronize(s));
  }
  const int nc = L.nc;
  // contracted boxes (begin and end on each contracted leg, pair order) -> ids
  auto coord = [&](int64_t e, int k, int w) -> int64_t {
    const bool onB = e >= na;
    const tq_bs *T = onB ? B : A;
    const int64_t blk = onB ? e - na : e;
    const int leg = onB ? L.bl[k] : L.al[k];
    return (w ? T->h_end : T->h_begin)[blk * T->rank + leg];
  };
  auto box_less = [&](int64_t x, int64_t y) {
    for (int k = 0; k < nc; k++)
      for (int w = 0; w < 2; w++) {
        const int64_t a = coord(x, k, w), b = coord(y, k, w);
        if (a != b) return a < b;
      }
    return false;
  };
  std::vector<int64_t> ord((size_t)(na + nbk));
  for (int64_t e = 0; e < na + nbk; e++) ord[e] = e;
  std::sort(ord.begin(), ord.end(), box_less);
  std::vector<int32_t> boxid((size_t)(na + nbk));
  std::vector<uint8_t> onA, onB;
  int32_t nboxes = 0;
  for (size_t q = 0; q < ord.size(); q++) {
    if (q == 0 || box_less(ord[q - 1], ord[q])) {
      nboxes++;
      onA.push_back(0);
      onB.push_back(0);
    }
    boxid[ord[q]] = nboxes - 1;
    (ord[q] < na ? onA : onB)[nboxes - 1] = 1;
  }
  // signature of every free box: its blocks' matched contracted boxes, sorted
  typedef std::pair<int32_t, int32_t> BoxBlk;  // (box id, block)
  std::vector<std::vector<BoxBlk>> sigA((size_t)KA), sigB((size_t)KB);
  for (int64_t i = 0; i < na; i++)
    if (onA[boxid[i]] && onB[boxid[i]]) sigA[keyA[i]].push_back(BoxBlk(boxid[i], (int32_t)i));
  for (int64_t j = 0; j < nbk; j++)
    if (onA[boxid[na + j]] && onB[boxid[na + j]])
      sigB[keyB[j]].push_back(BoxBlk(boxid[na + j], (int32_t)j));
  std::map<std::vector<int32_t>, int32_t> cmap;
  std::vector<int32_t> clsA((size_t)KA, -1), clsB((size_t)KB, -1);
  std::vector<std::vector<int32_t>> cboxes;
  auto classify = [&](std::vector<std::vector<BoxBlk>> &sig, std::vector<int32_t> &cls) {
    for (size_t x = 0; x < sig.size(); x++) {
      if (sig[x].empty()) continue;
      std::sort(sig[x].begin(), sig[x].end());
      std::vector<int32_t> ids;
      for (size_t q = 0; q < sig[x].size(); q++) {
        if (q && sig[x][q].first == sig[x][q - 1].first) return false;  // a box twice
        ids.push_back(sig[x][q].first);
      }
      auto f = cmap.find(ids);
      if (f == cmap.end()) {
        f = cmap.emplace(ids, (int32_t)cboxes.size()).first;
        cboxes.push_back(ids);
      }
      cls[x] = f->second;
    }
    return true;
  };
  if (!classify(sigA, clsA) || !classify(sigB, clsB)) return TQ_OK;
  // every matched box belongs to one class, the same on both sides
  std::vector<int32_t> bcA((size_t)nboxes, -1), bcB((size_t)nboxes, -1);
  auto box_classes = [&](const std::vector<std::vector<BoxBlk>> &sig,
                         const std::vector<int32_t> &cls, std::vector<int32_t> &bc) {
    for (size_t x = 0; x < sig.size(); x++)
      for (const BoxBlk &e : sig[x]) {
        if (bc[e.first] >= 0 && bc[e.first] != cls[x]) return false;
        bc[e.first] = cls[x];
      }
    return true;
  };
  if (!box_classes(sigA, clsA, bcA) || !box_classes(sigB, clsB, bcB)) return TQ_OK;
  for (int32_t b = 0; b < nboxes; b++)
    if (bcA[b] != bcB[b]) return TQ_OK;
  const int64_t ncls = (int64_t)cboxes.size();
  // members of each class (free boxes in key order) and their sizes
  auto free_size = [&](const tq_bs *T, int64_t blk, int32_t nf, const int32_t *fl) {
    int64_t m = 1;
    for (int q = 0; q < nf; q++)
      m *= T->h_end[blk * T->rank + fl[q]] - T->h_begin[blk * T->rank + fl[q]] + 1;
    return m;
  };
  std::vector<std::vector<int64_t>> memX((size_t)ncls), memY((size_t)ncls);
  std::vector<int64_t> posX((size_t)KA, -1), posY((size_t)KB, -1), mX((size_t)KA, 0),
      nY((size_t)KB, 0);
  for (int64_t i = 0; i < na; i++) mX[keyA[i]] = free_size(A, i, L.nfa, L.fa);
  for (int64_t j = 0; j < nbk; j++) nY[keyB[j]] = free_size(B, j, L.nfb, L.fb);
  for (int64_t x = 0; x < KA; x++)
    if (clsA[x] >= 0) {
      posX[x] = (int64_t)memX[clsA[x]].size();
      memX[clsA[x]].push_back(x);
    }
  for (int64_t y = 0; y < KB; y++)
    if (clsB[y] >= 0) {
      posY[y] = (int64_t)memY[clsB[y]].size();
      memY[clsB[y]].push_back(y);
    }
  // contracted extent of every box, and k-steps
  std::vector<int64_t> kbox((size_t)nboxes, 1);
  for (int64_t e = 0; e < na + nbk; e++) {
    int64_t k = 1;
    for (int q = 0; q < nc; q++) k *= coord(e, q, 1) - coord(e, q, 0) + 1;
    kbox[boxid[e]] = k;
  }
  // output block offsets per class and (A box, B box); every pair must be an
  // output block whose pairs are all the boxes of the class
  std::vector<int64_t> offs_base((size_t)ncls + 1, 0);
  for (int64_t c = 0; c < ncls; c++)
    offs_base[c + 1] = offs_base[c] + (int64_t)memX[c].size() * (int64_t)memY[c].size();
  if (offs_base[ncls] != no) return TQ_OK;
  std::vector<int64_t> offs((size_t)no, -1);
  for (int64_t o = 0; o < no; o++) {
    const int64_t x = xy[3 * o], y = xy[3 * o + 1], cnt = xy[3 * o + 2];
    const int32_t c = clsA[x];
    if (c < 0 || clsB[y] != c || cnt != (int64_t)cboxes[c].size()) return TQ_OK;
    int64_t &slot = offs[offs_base[c] + posX[x] * (int64_t)memY[c].size() + posY[y]];
    if (slot >= 0) return TQ_OK;
    slot = P->C->h_offsets[o];
  }
  // the layout: virtual rows / columns, slice storage, slicing work items
  std::vector<int64_t> rowA((size_t)KA, 0), rowB((size_t)KB, 0);
  std::vector<OzRowMap> rmA, rmB;
  std::vector<OzClassItem> itA, itB;
  std::vector<int32_t> blkA, blkB;
  std::vector<OzClassOut> out((size_t)ncls);
  const int32_t pack = oz_pack_of(sl, A->dtype == TQ_F16);
  const int64_t kw = oz_kstep_cols(A->dtype == TQ_F16, pack);
  const int64_t se = (int64_t)sl * pack;  // slices per stored step
  std::vector<int64_t> tstart((size_t)ncls + 1, 0), ksum((size_t)ncls);
  std::vector<OzPairRec> prs((size_t)ncls);
  int64_t unitA = 0, unitB = 0, vA = 0, vB = 0;
  for (int64_t c = 0; c < ncls; c++) {
    const std::vector<int32_t> &bx = cboxes[c];
    const int32_t nbox = (int32_t)bx.size();
    std::vector<int32_t> koff(nbox), nk(nbox);
    int64_t ks = 0;
    for (int32_t q = 0; q < nbox; q++) {
      koff[q] = (int32_t)ks;
      nk[q] = (int32_t)((kbox[bx[q]] + kw - 1) / kw);
      ks += nk[q];
    }
    if (ks > 0x7fffffff) return TQ_OK;
    ksum[c] = ks;
    const int64_t nYc = (int64_t)memY[c].size();
    // side A: 128-row tiles
    const int64_t r0 = vA, bbA = (int64_t)blkA.size();
    for (size_t xi = 0; xi < memX[c].size(); xi++) {
      const int64_t x = memX[c][xi];
      rowA[x] = vA;
      for (int64_t r = 0; r < mX[x]; r++)
        rmA.push_back(OzRowMap{offs_base[c] + (int64_t)xi * nYc, (int32_t)xi, (int32_t)r,
                               (int32_t)mX[x], 0});
      vA += mX[x];
      for (int32_t q = 0; q < nbox; q++) blkA.push_back(sigA[x][q].second);
    }
    const int64_t Mc = vA - r0, tmA = (Mc + OZ_M - 1) / OZ_M;
    const int64_t u0A = unitA;
    for (int64_t rt = 0; rt < tmA; rt++) {
      const int32_t rows = (int32_t)std::min<int64_t>(OZ_M, Mc - rt * OZ_M);
      for (int32_t q = 0; q < nbox; q++)
        itA.push_back(OzClassItem{u0A + rt * ks * se * (OZ_M / 8), r0 + rt * OZ_M, bbA, koff[q],
                                  nk[q], rows, q, nbox, 0});
      unitA += ks * se * ((rows + 7) / 8);
    }
    // side B: tile-width column tiles
    const int64_t c0 = vB, bbB = (int64_t)blkB.size();
    for (size_t yi = 0; yi < memY[c].size(); yi++) {
      const int64_t y = memY[c][yi];
      rowB[y] = vB;
      for (int64_t r = 0; r < nY[y]; r++)
        rmB.push_back(OzRowMap{0, (int32_t)yi, (int32_t)r, (int32_t)nY[y], 0});
      vB += nY[y];
      for (int32_t q = 0; q < nbox; q++) blkB.push_back(sigB[y][q].second);
    }
    const int64_t Nc = vB - c0, tmB = (Nc + tn - 1) / tn;
    const int64_t u0B = unitB;
    for (int64_t ct = 0; ct < tmB; ct++) {
      const int32_t rows = (int32_t)std::min<int64_t>(tn, Nc - ct * tn);
      for (int32_t q = 0; q < nbox; q++)
        itB.push_back(OzClassItem{u0B + ct * ks * se * (tn / 8), c0 + ct * tn, bbB, koff[q],
                                  nk[q], rows, q, nbox, 0});
      unitB += ks * se * ((rows + 7) / 8);
    }
    out[c] = OzClassOut{Mc, Nc, r0, c0};
    tstart[c + 1] = tstart[c] + tmA * tmB;
    prs[c] = OzPairRec{256 * u0A, 256 * u0B, (int32_t)ks, 0};
  }
  // free boxes outside every class keep exponent rows (the exponent pass covers
  // all blocks) after the class rows
  for (int64_t x = 0; x < KA; x++)
    if (clsA[x] < 0) rowA[x] = vA, vA += mX[x];
  for (int64_t y = 0; y < KB; y++)
    if (clsB[y] < 0) rowB[y] = vB, vB += nY[y];
  if (vA != nexpA || vB != nexpB)
    return fail(TQ_ERR_CUDA, "inconsistent class layout (exponent rows)");
  TQ_CHECK(upload(P->rowA, rowA, s));
  TQ_CHECK(upload(P->rowB, rowB, s));
  TQ_CHECK(upload(P->rmapA, rmA, s));
  TQ_CHECK(upload(P->rmapB, rmB, s));
  TQ_CHECK(upload(P->itemsA, itA, s));
  TQ_CHECK(upload(P->itemsB, itB, s));
  TQ_CHECK(upload(P->blkA, blkA, s));
  TQ_CHECK(upload(P->blkB, blkB, s));
  TQ_CHECK(upload(P->cls_out, out, s));
  TQ_CHECK(upload(P->cls_offs, offs, s));
  TQ_CHECK(upload(P->tc_tile_start, tstart, s));
  TQ_CHECK(upload(P->ksum, ksum, s));
  TQ_CHECK(upload(P->pair_tab, prs, s));
  TQ_CHECK(P->expA.alloc(std::max<int64_t>(nexpA, 1), s));
  TQ_CHECK(P->expB.alloc(std::max<int64_t>(nexpB, 1), s));
  TQ_CHECK(P->sliceA.alloc(std::max<int64_t>(unitA, 1) * 256, s));
  TQ_CHECK(P->sliceB.alloc(std::max<int64_t>(unitB, 1) * 256, s));
  P->classes = true;
  P->n_cls = ncls;
  P->tc_tiles = tstart[ncls];
  P->hyb_tiles = 0;
  P->tilesA = (int64_t)itA.size();
  P->tilesB = (int64_t)itB.size();
  P->tc_side[0] = make_side(A, L.nfa, L.fa, L.nc, L.al, P->keyA.p, P->rowA.p, P->rowstartA.p,
                            P->tilestartA.p, P->unitA.p);
  P->tc_side[1] = make_side(B, L.nfb, L.fb, L.nc, L.bl, P->keyB.p, P->rowB.p, P->rowstartB.p,
                            P->tilestartB.p, P->unitB.p);
  P->tc_side[0].pack = P->tc_side[1].pack = oz_pack_of(sl, A->dtype == TQ_F16);
  const int64_t n_rows[2] = {P->rowsA, P->rowsB}, n_items[2] = {P->tilesA, P->tilesB},
                n_exps[2] = {nexpA, nexpB};
  int32_t *exps[2] = {P->expA.p, P->expB.p};
  uint8_t *slices[2] = {P->sliceA.p, P->sliceB.p};
  const OzClassItem *items[2] = {P->itemsA.p, P->itemsB.p};
  const OzRowMap *rmaps[2] = {P->rmapA.p, P->rmapB.p};
  const int32_t *blks[2] = {P->blkA.p, P->blkB.p};
  for (int k = 0; k < 2; k++) {
    OzSide &S = P->tc_side[k];
    S.exps = exps[k];
    S.slices = slices[k];
    S.n_rows = n_rows[k];
    S.n_tiles = n_items[k];
    S.n_exps = n_exps[k];
    S.s = sl;
    S.rt_rows = k == 0 ? OZ_M : tn;
    S.items = items[k];
    S.rmap = rmaps[k];
    S.blk = blks[k];
  }
  OzJob &J = P->tc_job;
  J = OzJob{};
  P->out = nullptr;  // a rebuilt job array writes the result tensor's buffer
  J.g = make_gemm_job(P);
  J.f16 = P->A->dtype == TQ_F16;
  J.pack = oz_pack_of(sl, J.f16);
  J.prs = P->pair_tab.p;
  J.tile_start = P->tc_tile_start.p;
  J.n_tiles = P->tc_tiles;
  J.ksum = P->ksum.p;
  J.sliceA = P->sliceA.p;
  J.sliceB = P->sliceB.p;
  J.keyA = P->keyA.p;
  J.keyB = P->keyB.p;
  J.rowA = P->rowA.p;
  J.rowB = P->rowB.p;
  J.expA = P->expA.p;
  J.expB = P->expB.p;
  J.s = sl;
  J.tile_n = tn;
  J.cls = P->cls_out.p;
  J.n_cls = ncls;
  J.rmapA = P->rmapA.p;
  J.rmapB = P->rmapB.p;
  J.offs = P->cls_offs.p;
  *used = true;
  return oz_batch_build({J}, {P->tc_side[0], P->tc_side[1]}, s, P->tcb);
}

static tq_status plan_tc(tq_plan *P, int64_t KA, int64_t KB, cudaStream_t s) {
  const LegSpec &L = P->L;
  const tq_bs *A = P->A, *B = P->B;
  int32_t sl = P->opts.slices;
  if (P->opts.precision == TQ_PREC_TENSOR) {
    // binary16 operands go to the tensor cores as they are, four 16-column
    // k-steps packed per step
    if (sl > 1) return fail(TQ_ERR_INVALID, "the tensor form has no slices");
    sl = OZ_F16_PACK;
  }
  if (sl == 0) sl = P->opts.precision == TQ_PREC_OZAKI ? 5 : 3;
  if (P->opts.precision != TQ_PREC_TENSOR && (sl < 1 || sl > OZ_MAXS))
    return fail(TQ_ERR_INVALID, "slice count outside 1..7");
  P->slices = sl;
  const int32_t tn = P->opts.tile_n ? P->opts.tile_n : OZ_N;
  if (tn != 32 && tn != 64 && tn != 96) return fail(TQ_ERR_INVALID, "tile width must be 32, 64 or 96");
  if (P->opts.native_fill < 0 || P->opts.native_fill > 1000)
    return fail(TQ_ERR_INVALID, "native_fill outside 0..1000");
  P->tile_n = tn;
  P->classes = false;
  P->n_cls = 0;
  P->tc_job = OzJob{};
  if (KA > (1 << 26) || KB > (1 << 26))
    return fail(TQ_ERR_UNSUPPORTED, "too many distinct free boxes for the sliced forms");
  const int64_t np = P->n_pairs, no = P->n_out;
  DevArray<int32_t> bad;
  TQ_CHECK(bad.alloc(1, s));
  TQ_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
  count_launch(), tc_align_kernel<<<nblk(np), 256, 0, s>>>(A->view(), B->view(), L, P->pa.p, P->pb.p, np, bad.p);
  TQ_CUDA(cudaGetLastError());
  // per-block geometry of both sides
  DevArray<int64_t> mkA, mkB, rA, rB, tA, tB, uA, uB, tiles, tot;
  TQ_CHECK(mkA.alloc(KA, s));
  TQ_CHECK(mkB.alloc(KB, s));
  TQ_CUDA(cudaMemsetAsync(mkA.p, 0, KA * 8, s));
  TQ_CUDA(cudaMemsetAsync(mkB.p, 0, KB * 8, s));
  TQ_CHECK(rA.alloc(A->nb, s));
  TQ_CHECK(tA.alloc(A->nb, s));
  TQ_CHECK(uA.alloc(A->nb, s));
  TQ_CHECK(rB.alloc(B->nb, s));
  TQ_CHECK(tB.alloc(B->nb, s));
  TQ_CHECK(uB.alloc(B->nb, s));
  TQ_CHECK(tot.alloc(10, s));
  const bool f16 = A->dtype == TQ_F16;
  const int32_t pack = oz_pack_of(sl, f16);
  OzSide SA = make_side(A, L.nfa, L.fa, L.nc, L.al, P->keyA.p, nullptr, nullptr, nullptr, nullptr);
  OzSide SB = make_side(B, L.nfb, L.fb, L.nc, L.bl, P->keyB.p, nullptr, nullptr, nullptr, nullptr);
  SA.pack = SB.pack = pack;
  count_launch(), tc_block_stats_kernel<<<nblk(A->nb), 256, 0, s>>>(SA, OZ_M, sl, mkA.p, rA.p, tA.p, uA.p);
  count_launch(), tc_block_stats_kernel<<<nblk(B->nb), 256, 0, s>>>(SB, tn, sl, mkB.p, rB.p, tB.p, uB.p);
  TQ_CUDA(cudaGetLastError());
  TQ_CHECK(P->rowstartA.alloc(A->nb, s));
  TQ_CHECK(P->tilestartA.alloc(A->nb, s));
  TQ_CHECK(P->unitA.alloc(A->nb, s));
  TQ_CHECK(P->rowstartB.alloc(B->nb, s));
  TQ_CHECK(P->tilestartB.alloc(B->nb, s));
  TQ_CHECK(P->unitB.alloc(B->nb, s));
  TQ_CHECK(P->rowA.alloc(KA, s));
  TQ_CHECK(P->rowB.alloc(KB, s));
  TQ_CHECK(scan_exclusive(rA.p, P->rowstartA.p, A->nb, tot.p + 0, s));
  TQ_CHECK(scan_exclusive(tA.p, P->tilestartA.p, A->nb, tot.p + 1, s));
  TQ_CHECK(scan_exclusive(uA.p, P->unitA.p, A->nb, tot.p + 2, s));
  TQ_CHECK(scan_exclusive(mkA.p, P->rowA.p, KA, tot.p + 3, s));
  TQ_CHECK(scan_exclusive(rB.p, P->rowstartB.p, B->nb, tot.p + 4, s));
  TQ_CHECK(scan_exclusive(tB.p, P->tilestartB.p, B->nb, tot.p + 5, s));
  TQ_CHECK(scan_exclusive(uB.p, P->unitB.p, B->nb, tot.p + 6, s));
  TQ_CHECK(scan_exclusive(mkB.p, P->rowB.p, KB, tot.p + 7, s));
  // per-output tiles and k-steps
  TQ_CHECK(P->nk_pair.alloc(np, s));
  TQ_CHECK(P->ksum.alloc(no, s));
  TQ_CHECK(tiles.alloc(no, s));
  TQ_CHECK(P->tc_tile_start.alloc(no + 1, s));
  DevArray<int64_t> nt_native;
  TQ_CHECK(nt_native.alloc(no, s));
  TQ_CHECK(P->hyb_tile_start.alloc(no + 1, s));
  count_launch(), tc_out_kernel<<<nblk(no), 256, 0, s>>>(A->view(), B->view(), L, P->pa.p, P->pb.p, P->seg.p,
                                          P->perm.p, no, tn, P->opts.native_fill,
                                          (int32_t)oz_kstep_cols(f16, pack),
                                          P->nk_pair.p, tiles.p, P->ksum.p, nt_native.p);
  TQ_CUDA(cudaGetLastError());
  TQ_CHECK(scan_exclusive(tiles.p, P->tc_tile_start.p, no, tot.p + 8, s));
  TQ_CHECK(scan_exclusive(nt_native.p, P->hyb_tile_start.p, no, tot.p + 9, s));
  int64_t h[10];
  int32_t h_bad = 0;
  TQ_CUDA(cudaMemcpyAsync(h, tot.p, 10 * 8, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaMemcpyAsync(&h_bad, bad.p, 4, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  if (h_bad)
    return fail(TQ_ERR_UNSUPPORTED,
                "the sliced forms need sector-aligned blocks: matched blocks must cover the same "
                "interval on every contracted leg; use the native precision");
  P->rowsA = h[0];
  P->tilesA = h[1];
  P->nexpA = h[3];
  P->rowsB = h[4];
  P->tilesB = h[5];
  P->nexpB = h[7];
  bool classes = false;
  TQ_CHECK(plan_tc_classes(P, sl, tn, P->nexpA, P->nexpB, s, &classes));
  if (classes) return TQ_OK;
  P->tc_tiles = h[8];
  P->hyb_tiles = h[9];
  if (P->hyb_tiles < 0 || P->hyb_tiles > P->n_tiles)
    return fail(TQ_ERR_CUDA, "inconsistent block grouping (native tiles above the plan's)");
  TQ_CHECK(native_work(P, nt_native.p, P->hyb_tile_start.p, P->hyb_tiles, P->hyb, s));
  TQ_CHECK(P->expA.alloc(std::max<int64_t>(P->nexpA, 1), s));
  TQ_CHECK(P->expB.alloc(std::max<int64_t>(P->nexpB, 1), s));
  TQ_CHECK(P->sliceA.alloc(std::max<int64_t>(h[2], 1) * 256, s));
  TQ_CHECK(P->sliceB.alloc(std::max<int64_t>(h[6], 1) * 256, s));
  // this contraction as a batch of one job with two operand sides
  P->tc_side[0] = make_side(A, L.nfa, L.fa, L.nc, L.al, P->keyA.p, P->rowA.p, P->rowstartA.p,
                            P->tilestartA.p, P->unitA.p);
  P->tc_side[1] = make_side(B, L.nfb, L.fb, L.nc, L.bl, P->keyB.p, P->rowB.p, P->rowstartB.p,
                            P->tilestartB.p, P->unitB.p);
  P->tc_side[0].pack = P->tc_side[1].pack = oz_pack_of(sl, A->dtype == TQ_F16);
  const int64_t n_rows[2] = {P->rowsA, P->rowsB}, n_tiles[2] = {P->tilesA, P->tilesB},
                n_exps[2] = {P->nexpA, P->nexpB};
  int32_t *exps[2] = {P->expA.p, P->expB.p};
  uint8_t *slices[2] = {P->sliceA.p, P->sliceB.p};
  for (int k = 0; k < 2; k++) {
    OzSide &S = P->tc_side[k];
    S.exps = exps[k];
    S.slices = slices[k];
    S.n_rows = n_rows[k];
    S.n_tiles = n_tiles[k];
    S.n_exps = n_exps[k];
    S.s = sl;
    S.rt_rows = k == 0 ? OZ_M : tn;
  }
  OzJob &J = P->tc_job;
  P->out = nullptr;  // a rebuilt job array writes the result tensor's buffer
  J.g = make_gemm_job(P);
  J.f16 = P->A->dtype == TQ_F16;
  J.pack = oz_pack_of(sl, J.f16);
  J.tile_start = P->tc_tile_start.p;
  J.n_tiles = P->tc_tiles;
  J.ksum = P->ksum.p;
  J.nk_pair = P->nk_pair.p;
  J.sliceA = P->sliceA.p;
  J.sliceB = P->sliceB.p;
  J.unitA = P->unitA.p;
  J.unitB = P->unitB.p;
  J.keyA = P->keyA.p;
  J.keyB = P->keyB.p;
  J.rowA = P->rowA.p;
  J.rowB = P->rowB.p;
  J.expA = P->expA.p;
  J.expB = P->expB.p;
  J.s = sl;
  J.tile_n = tn;
  TQ_CHECK(P->pair_tab.alloc(std::max<int64_t>(np, 1), s));
  J.prs = P->pair_tab.p;
  TQ_CHECK(oz_pair_table(J, np, P->pair_tab.p, s));
  return oz_batch_build({J}, {P->tc_side[0], P->tc_side[1]}, s, P->tcb);
}

// The output blocks that block grouping sent to plain FP64 (after the sliced
// launch; the two write disjoint output blocks).
tq_status run_hybrid_native(tq_plan *P, cudaStream_t s) {
  if (!P->tc || P->hyb_tiles == 0) return TQ_OK;
  GemmJob job = make_gemm_job(P);
  job.tile_start = P->hyb_tile_start.p;
  return launch_gemm_native(job, P->hyb_tiles, P->A->dtype, s, &P->hyb.w);
}

static tq_status run_tc(tq_plan *P, cudaStream_t s) {
  if (P->tc_tiles) {
    NvtxRange r("tq_prepare");
    TQ_CHECK(oz_batch_prepare(P->tcb, s));
  }
  if (P->profile) TQ_CUDA(cudaEventRecord(P->ev[1], s));
  NvtxRange r("tq_gemm");
  if (P->tc_tiles) TQ_CHECK(oz_batch_gemm(P->tcb, s));
  return run_hybrid_native(P, s);
}

// The sliced forms take float64 tensors; the tensor form takes binary16 ones.
static tq_status check_precision(int32_t precision, tq_dtype dtype) {
  if (precision != TQ_PREC_NATIVE && precision != TQ_PREC_OZAKI && precision != TQ_PREC_BF16X3 &&
      precision != TQ_PREC_TENSOR)
    return fail(TQ_ERR_INVALID, "unknown precision");
  if ((precision == TQ_PREC_OZAKI || precision == TQ_PREC_BF16X3) && dtype != TQ_F64)
    return fail(TQ_ERR_UNSUPPORTED, "the sliced tensor-core forms take float64 tensors");
  if (precision == TQ_PREC_TENSOR && dtype != TQ_F16)
    return fail(TQ_ERR_UNSUPPORTED, "the tensor form takes half tensors");
  return TQ_OK;
}

tq_status validate_legs(const tq_bs *A, const tq_bs *B, int32_t n_legs, const int64_t *a_legs,
                        const int64_t *b_legs, LegSpec &L) {
  if (!A || !B) return fail(TQ_ERR_INVALID, "tensor is NULL");
  if (A->dtype != B->dtype) return fail(TQ_ERR_INVALID, "tensors have different dtypes");
  if (n_legs < 0 || n_legs > TQ_MAXR) return fail(TQ_ERR_INVALID, "bad number of contracted legs");
  if (n_legs && (!a_legs || !b_legs)) return fail(TQ_ERR_INVALID, "leg lists are NULL");
  std::memset(&L, 0, sizeof(L));
  L.nc = n_legs;
  L.rank_a = A->rank;
  L.rank_b = B->rank;
  bool used_a[TQ_MAXR] = {false}, used_b[TQ_MAXR] = {false};
  for (int32_t k = 0; k < n_legs; k++) {
    if (a_legs[k] < 0 || a_legs[k] >= A->rank || b_legs[k] < 0 || b_legs[k] >= B->rank)
      return fail(TQ_ERR_INVALID, "contracted leg index out of range");
    if (used_a[a_legs[k]] || used_b[b_legs[k]])
      return fail(TQ_ERR_INVALID, "a leg is contracted twice");
    used_a[a_legs[k]] = used_b[b_legs[k]] = true;
    if (A->dimension[a_legs[k]] != B->dimension[b_legs[k]])
      return fail(TQ_ERR_INVALID, "The dimensions from two tensors to be contracted do not match");
    L.al[k] = (int32_t)a_legs[k];
    L.bl[k] = (int32_t)b_legs[k];
  }
  for (int32_t l = 0; l < A->rank; l++)
    if (!used_a[l]) L.fa[L.nfa++] = l;
  for (int32_t l = 0; l < B->rank; l++)
    if (!used_b[l]) L.fb[L.nfb++] = l;
  return TQ_OK;
}

// structure_only: the symbolic stage alone (pairs, output boxes, offsets); the
// result's data are not allocated and no work list is built, so the plan and
// its result are for reading the block list only and never leave the library.
tq_status plan_build(const tq_bs *A, const tq_bs *B, int32_t n_legs, const int64_t *a_legs,
                     const int64_t *b_legs, const tq_contract_opts *opts, cudaStream_t s,
                     tq_plan **plan_out, tq_bs **out, bool structure_only = false) {
  NvtxRange range("tq_plan");
  LegSpec L;
  TQ_CHECK(validate_legs(A, B, n_legs, a_legs, b_legs, L));
  tq_contract_opts o = {TQ_PREC_NATIVE, TQ_LAYOUT_REFERENCE, 0, 0, 0, 0};
  if (opts) o = *opts;
  TQ_CHECK(check_precision(o.precision, A->dtype));
  if (o.layout != TQ_LAYOUT_REFERENCE && o.layout != TQ_LAYOUT_REDUCED)
    return fail(TQ_ERR_INVALID, "unknown layout");
  TQ_CHECK(sync_device_meta(const_cast<tq_bs *>(A), s));
  TQ_CHECK(sync_device_meta(const_cast<tq_bs *>(B), s));

  std::unique_ptr<tq_plan> P(new tq_plan());
  P->A = A;
  P->B = B;
  P->L = L;
  P->opts = o;
  const int32_t rc = L.nfa + L.nfb;
  std::vector<int64_t> new_dim;
  for (int q = 0; q < L.nfa; q++) new_dim.push_back(A->dimension[L.fa[q]]);
  for (int q = 0; q < L.nfb; q++) new_dim.push_back(B->dimension[L.fb[q]]);
  if (rc > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "result rank above 12");
  const DevBS Av = A->view(), Bv = B->view();

  // 1. pairs
  DevArray<int64_t> counts, row_off, tot;
  TQ_CHECK(counts.alloc(std::max<int64_t>(A->nb, 1), s));
  TQ_CHECK(row_off.alloc(std::max<int64_t>(A->nb, 1), s));
  TQ_CHECK(tot.alloc(4, s));
  TQ_CHECK(match_pairs(Av, Bv, L, counts.p, s));
  TQ_CHECK(scan_exclusive(counts.p, row_off.p, A->nb, tot.p, s));
  int64_t n_pairs = 0;
  TQ_CUDA(cudaMemcpyAsync(&n_pairs, tot.p, 8, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  if (n_pairs > 0x7fffffffLL) return fail(TQ_ERR_UNSUPPORTED, "more than 2^31 block pairs");
  P->n_pairs = n_pairs;
  TQ_CHECK(P->pa.alloc(std::max<int64_t>(n_pairs, 1), s));
  TQ_CHECK(P->pb.alloc(std::max<int64_t>(n_pairs, 1), s));
  TQ_CHECK(emit_pairs(Av, Bv, L, row_off.p, P->pa.p, P->pb.p, s));

  // per-pair work (m*n*k) for the flop count; dot chunks for rank-0 results
  DevArray<int64_t> mnk, mnk_off;
  TQ_CHECK(mnk.alloc(std::max<int64_t>(n_pairs, 1), s));
  TQ_CHECK(mnk_off.alloc(std::max<int64_t>(n_pairs, 1), s));
  DevArray<int64_t> chunks;
  if (rc == 0) {
    TQ_CHECK(chunks.alloc(std::max<int64_t>(n_pairs, 1), s));
    TQ_CHECK(P->chunk_start.alloc(std::max<int64_t>(n_pairs, 1), s));
  }
  if (n_pairs) {
    count_launch(), pair_stats_kernel<<<nblk(n_pairs), 256, 0, s>>>(Av, Bv, L, P->pa.p, P->pb.p, n_pairs, mnk.p,
                                                     rc == 0 ? chunks.p : nullptr);
    TQ_CUDA(cudaGetLastError());
  }
  TQ_CHECK(scan_exclusive(mnk.p, mnk_off.p, n_pairs, tot.p + 1, s));

  tq_bs *C = new_tensor(A->dtype, rc, new_dim.data());
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> Cguard(C, tq_bs_destroy);
  P->C = C;  // borrowed until the plan is handed out; Cguard owns it on failure

  if (rc == 0) {
    // rank-0 result: one scalar, sum over all pairs
    TQ_CHECK(scan_exclusive(chunks.p, P->chunk_start.p, n_pairs, tot.p + 2, s));
    int64_t h[3] = {0, 0, 0};
    TQ_CUDA(cudaMemcpyAsync(h, tot.p, 24, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaStreamSynchronize(s));
    P->flops = 2.0 * (double)h[1];
    P->n_chunks = h[2];
    TQ_CHECK(P->partials.alloc(std::max<int64_t>(P->n_chunks, 1), s));
    TQ_CHECK(alloc_data(C, 1, s));
    C->nb = 0;
    C->host_valid = true;
    C->dev_valid = true;
    P->n_out = 0;
  } else {
    int64_t n_out = n_pairs;
    P->tc = o.precision != TQ_PREC_NATIVE;
    int64_t KA = 1, KB = 1;
    if ((o.layout == TQ_LAYOUT_REDUCED || P->tc) && n_pairs) {
      // interval-id keys of the free boxes: output grouping and exponent classes
      TQ_CHECK(P->keyA.alloc(std::max<int64_t>(A->nb, 1), s));
      TQ_CHECK(P->keyB.alloc(std::max<int64_t>(B->nb, 1), s));
      TQ_CHECK(box_keys(A, L.nfa, L.fa, P->keyA.p, &KA, s));
      TQ_CHECK(box_keys(B, L.nfb, L.fb, P->keyB.p, &KB, s));
    }
    if (o.layout == TQ_LAYOUT_REDUCED && n_pairs) {
      // 3. group pairs by output box
      DevArray<int64_t> key, flag, sid;
      if (KB > 0 && KA > (int64_t(1) << 62) / KB)
        return fail(TQ_ERR_UNSUPPORTED, "output box key range exceeds 2^62");
      TQ_CHECK(key.alloc(n_pairs, s));
      TQ_CHECK(P->perm.alloc(n_pairs, s));
      count_launch(), pair_key_kernel<<<nblk(n_pairs), 256, 0, s>>>(P->pa.p, P->pb.p, n_pairs, P->keyA.p,
                                                    P->keyB.p, KA, key.p);
      count_launch(), iota_kernel<<<nblk(n_pairs), 256, 0, s>>>(P->perm.p, n_pairs);
      TQ_CUDA(cudaGetLastError());
      TQ_CHECK(radix_sort_pairs(key.p, P->perm.p, n_pairs, bits_for(KA * KB), s));
      TQ_CHECK(flag.alloc(n_pairs, s));
      TQ_CHECK(sid.alloc(n_pairs, s));
      count_launch(), seg_flag_kernel<<<nblk(n_pairs), 256, 0, s>>>(key.p, n_pairs, flag.p);
      TQ_CHECK(scan_exclusive(flag.p, sid.p, n_pairs, tot.p + 3, s));
      TQ_CUDA(cudaMemcpyAsync(&n_out, tot.p + 3, 8, cudaMemcpyDeviceToHost, s));
      TQ_CUDA(cudaStreamSynchronize(s));
      TQ_CHECK(P->seg.alloc(n_out + 1, s));
      count_launch(), seg_start_kernel<<<nblk(n_pairs), 256, 0, s>>>(flag.p, sid.p, n_pairs, n_out, P->seg.p);
      TQ_CUDA(cudaGetLastError());
    } else {
      TQ_CHECK(P->seg.alloc(n_pairs + 1, s));
      count_launch(), iota_kernel<<<nblk(n_pairs + 1), 256, 0, s>>>(P->seg.p, n_pairs + 1);
      TQ_CUDA(cudaGetLastError());
    }
    P->n_out = n_out;
    // 2. output metadata: boxes, strides, element counts, offsets; tiles
    C->nb = n_out;
    TQ_CHECK(C->d_meta.alloc(3 * (size_t)n_out * rc + n_out, s));
    DevArray<int64_t> n_elem, tiles;
    TQ_CHECK(n_elem.alloc(std::max<int64_t>(n_out, 1), s));
    TQ_CHECK(tiles.alloc(std::max<int64_t>(n_out, 1), s));
    TQ_CHECK(P->tile_start.alloc(n_out + 1, s));
    if (n_out) {
      int64_t *cb = C->d_meta.p, *ce = cb + n_out * rc, *cs = ce + n_out * rc;
      count_launch(), out_meta_kernel<<<nblk(n_out), 256, 0, s>>>(Av, Bv, L, P->pa.p, P->pb.p, P->seg.p,
                                                  P->perm.p, n_out, rc, cb, ce, cs, n_elem.p,
                                                  tiles.p);
      TQ_CUDA(cudaGetLastError());
    }
    int64_t *c_off = C->d_meta.p + 3 * n_out * rc;
    TQ_CHECK(scan_exclusive(n_elem.p, c_off, n_out, tot.p + 2, s));
    TQ_CHECK(scan_exclusive(tiles.p, P->tile_start.p, n_out, tot.p + 3, s));
    int64_t h[4] = {0, 0, 0, 0};
    TQ_CUDA(cudaMemcpyAsync(h, tot.p, 32, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaStreamSynchronize(s));
    P->flops = 2.0 * (double)h[1];
    P->n_tiles = h[3];
    if (structure_only) {
      C->n_elem = h[2];
      C->host_valid = false;
      C->dev_valid = true;
      P->C = C;
      Cguard.release();
      *out = C;
      *plan_out = P.release();
      return TQ_OK;
    }
    TQ_CHECK(alloc_data(C, h[2], s));
    TQ_CHECK(native_work(P.get(), tiles.p, P->tile_start.p, P->n_tiles, P->nat, s));
    C->host_valid = false;
    C->dev_valid = true;
    P->KA = KA;
    P->KB = KB;
    P->keys = (o.layout == TQ_LAYOUT_REDUCED || P->tc) && n_pairs;
    if (P->tc && n_pairs) TQ_CHECK(plan_tc(P.get(), KA, KB, s));
  }
  P->C = C;
  Cguard.release();
  *out = C;
  *plan_out = P.release();
  return TQ_OK;
}

// A new schedule (precision, slices, tile width, grouping) for a planned
// contraction: the symbolic stage is kept, only the tensor-core part is rebuilt.
tq_status plan_reschedule(tq_plan *P, const tq_contract_opts &o, cudaStream_t s) {
  TQ_CHECK(check_precision(o.precision, P->A->dtype));
  if (o.layout != P->opts.layout) return fail(TQ_ERR_INVALID, "a new schedule keeps the layout");
  const bool tc = o.precision != TQ_PREC_NATIVE && P->C->rank > 0 && P->n_pairs > 0;
  if (tc && !P->keys)
    return fail(TQ_ERR_INVALID,
                "plan was made for plain arithmetic in the reference layout; create it with a "
                "tensor-core precision or the reduced layout to reschedule it");
  // wait for launches that still read the old schedule's arrays
  TQ_CUDA(cudaStreamSynchronize(s));
  P->sched_gen++;
  P->opts = o;
  P->tc = o.precision != TQ_PREC_NATIVE;
  P->tc_tiles = P->hyb_tiles = 0;
  P->sched_ok = false;
  if (tc) TQ_CHECK(plan_tc(P, P->KA, P->KB, s));
  P->sched_ok = true;
  return TQ_OK;
}

// The tensor-core job array lives on the device: its output pointer is
// rewritten there (one thread), in stream order.
__global__ void set_job_output_kernel(OzJob *jobs, void *c) { jobs[0].g.C = c; }

// Points the numeric stage's writes at out (device-addressable), or back at
// the result tensor's buffer when out is null.
static tq_status plan_bind_output(tq_plan *P, void *out, cudaStream_t s) {
  if (P->out == out) return TQ_OK;
  P->out = out;
  if (P->tc && P->tcb.jobs.p) {
    count_launch(), set_job_output_kernel<<<1, 1, 0, s>>>(P->tcb.jobs.p, out ? out : P->C->data);
    TQ_CUDA(cudaGetLastError());
  }
  return TQ_OK;
}

static tq_status plan_run_to(tq_plan *P, void *out, cudaStream_t s);

tq_status plan_run(tq_plan *P, cudaStream_t s) { return plan_run_to(P, nullptr, s); }

static tq_status plan_run_to(tq_plan *P, void *out, cudaStream_t s) {
  if (!P->sched_ok)
    return fail(TQ_ERR_INVALID, "the plan's last reschedule failed; give it a valid schedule");
  TQ_CHECK(plan_bind_output(P, out, s));
  const GemmJob job = make_gemm_job(P);
  if (P->profile) TQ_CUDA(cudaEventRecord(P->ev[0], s));
  tq_status st = TQ_OK;
  if (P->C->rank == 0) {
    if (P->profile) TQ_CUDA(cudaEventRecord(P->ev[1], s));
    NvtxRange r("tq_gemm_native");
    st = launch_dot_native(job, P->n_pairs, P->chunk_start.p, P->n_chunks, P->partials.p,
                           P->A->dtype, s);
  } else if (P->tc && P->n_tiles) {
    st = run_tc(P, s);
  } else {
    if (P->profile) TQ_CUDA(cudaEventRecord(P->ev[1], s));
    NvtxRange r("tq_gemm_native");
    if (P->n_tiles) st = launch_gemm_native(job, P->n_tiles, P->A->dtype, s, &P->nat.w);
  }
  if (st == TQ_OK && P->profile) TQ_CUDA(cudaEventRecord(P->ev[2], s));
  return st;
}

tq_status plan_check(tq_plan *P, cudaStream_t s) {
  if (!P->tc || !P->tcb.err.p) return TQ_OK;
  return oz_batch_check(P->tcb, s);
}

}  // namespace tq

using namespace tq;

extern "C" {

tq_status tq_plan_create(const tq_bs *A, const tq_bs *B, int32_t n_legs, const int64_t *a_legs,
                         const int64_t *b_legs, const tq_contract_opts *opts, tq_stream stream,
                         tq_plan **plan, tq_bs **out) {
  if (!plan || !out) return fail(TQ_ERR_INVALID, "NULL output argument");
  return plan_build(A, B, n_legs, a_legs, b_legs, opts, (cudaStream_t)stream, plan, out);
}

tq_status tq_plan_execute(tq_plan *plan, tq_stream stream) {
  if (!plan) return fail(TQ_ERR_INVALID, "plan is NULL");
  return plan_run(plan, (cudaStream_t)stream);
}

tq_status tq_plan_execute_to(tq_plan *plan, void *dst, tq_memkind kind, tq_stream stream) {
  if (!plan || !dst) return fail(TQ_ERR_INVALID, "NULL argument");
  if (kind != TQ_MEM_HOST && kind != TQ_MEM_DEVICE) return fail(TQ_ERR_INVALID, "bad memory kind");
  cudaStream_t s = (cudaStream_t)stream;
  tq_plan *P = plan;
  void *dev = kind == TQ_MEM_DEVICE ? dst : nullptr;
  if (kind == TQ_MEM_HOST && P->C->rank > 0) {
    // page-locked host memory is addressable by the kernels (unified
    // addressing): they write it over the host link as they go
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, dst) == cudaSuccess && a.type == cudaMemoryTypeHost &&
        a.devicePointer)
      dev = a.devicePointer;
    else
      (void)cudaGetLastError();
  }
  if (dev) {
    TQ_CHECK(plan_run_to(P, dev, s));
    if (kind == TQ_MEM_HOST) TQ_CUDA(cudaStreamSynchronize(s));
    return TQ_OK;
  }
  // pageable host memory (or a rank-0 result): compute, then one copy
  TQ_CHECK(plan_run(P, s));
  return tq_bs_copy_data(P->C, dst, kind, stream);
}

tq_status tq_plan_reschedule(tq_plan *plan, const tq_contract_opts *opts, tq_stream stream) {
  if (!plan || !opts) return fail(TQ_ERR_INVALID, "NULL argument");
  return plan_reschedule(plan, *opts, (cudaStream_t)stream);
}

tq_status tq_plan_flops(const tq_plan *plan, double *flops, int64_t *n_pairs) {
  if (!plan) return fail(TQ_ERR_INVALID, "plan is NULL");
  if (flops) *flops = plan->flops;
  if (n_pairs) *n_pairs = plan->n_pairs;
  return TQ_OK;
}

tq_status tq_plan_destroy(tq_plan *plan) {
  delete plan;
  return TQ_OK;
}

tq_status tq_plan_set_profiling(tq_plan *plan, int32_t enable) {
  if (!plan) return fail(TQ_ERR_INVALID, "plan is NULL");
  if (enable)
    for (auto &e : plan->ev)
      if (!e) TQ_CUDA(cudaEventCreate(&e));
  plan->profile = enable != 0;
  return TQ_OK;
}

tq_status tq_plan_last_timings(tq_plan *plan, float *prepare_ms, float *gemm_ms) {
  if (!plan) return fail(TQ_ERR_INVALID, "plan is NULL");
  if (!plan->profile) return fail(TQ_ERR_INVALID, "profiling is off for this plan");
  TQ_CUDA(cudaEventSynchronize(plan->ev[2]));
  float a = 0.f, b = 0.f;
  TQ_CUDA(cudaEventElapsedTime(&a, plan->ev[0], plan->ev[1]));
  TQ_CUDA(cudaEventElapsedTime(&b, plan->ev[1], plan->ev[2]));
  if (prepare_ms) *prepare_ms = a;
  if (gemm_ms) *gemm_ms = b;
  return TQ_OK;
}

tq_status tq_plan_check(tq_plan *plan, tq_stream stream) {
  if (!plan) return fail(TQ_ERR_INVALID, "plan is NULL");
  return plan_check(plan, (cudaStream_t)stream);
}

tq_status tq_contract_blocks(const tq_bs *A, const tq_bs *B, int32_t n_legs,
                            const int64_t *a_legs, const int64_t *b_legs, int32_t layout,
                            int64_t cap, int64_t *n_blocks, int64_t *n_elem,
                            int64_t *begin_points, int64_t *end_points, int64_t *block_offsets,
                            int64_t *pair_a, int64_t *pair_b, tq_stream stream) {
  if (!A || !B || !n_blocks) return fail(TQ_ERR_INVALID, "NULL argument");
  if (cap < 0) return fail(TQ_ERR_INVALID, "negative capacity");
  if ((pair_a || pair_b) && layout != TQ_LAYOUT_REFERENCE)
    return fail(TQ_ERR_INVALID, "block pairs are one per output block only in the reference layout");
  cudaStream_t s = (cudaStream_t)stream;
  tq_contract_opts o = {TQ_PREC_NATIVE, layout, 0, 0, 0, 0};
  tq_plan *P = nullptr;
  tq_bs *C = nullptr;
  TQ_CHECK(plan_build(A, B, n_legs, a_legs, b_legs, &o, s, &P, &C, true));
  std::unique_ptr<tq_plan, tq_status (*)(tq_plan *)> Pg(P, tq_plan_destroy);
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> Cg(C, tq_bs_destroy);
  const int64_t nb = C->rank == 0 ? 0 : C->nb;
  *n_blocks = nb;
  if (n_elem) *n_elem = C->rank == 0 ? 1 : C->n_elem;
  if (cap < nb || nb == 0) return TQ_OK;
  TQ_CHECK(sync_host_meta(C, s));
  const size_t r = (size_t)C->rank;
  if (begin_points) std::copy(C->h_begin.begin(), C->h_begin.begin() + nb * r, begin_points);
  if (end_points) std::copy(C->h_end.begin(), C->h_end.begin() + nb * r, end_points);
  if (block_offsets) std::copy(C->h_offsets.begin(), C->h_offsets.begin() + nb, block_offsets);
  if (pair_a || pair_b) {
    std::vector<int32_t> h((size_t)nb);
    for (int side = 0; side < 2; side++) {
      int64_t *dst = side ? pair_b : pair_a;
      if (!dst) continue;
      TQ_CUDA(cudaMemcpyAsync(h.data(), side ? P->pb.p : P->pa.p, (size_t)nb * 4,
                              cudaMemcpyDeviceToHost, s));
      TQ_CUDA(cudaStreamSynchronize(s));
      for (int64_t q = 0; q < nb; q++) dst[q] = h[(size_t)q];
    }
  }
  return TQ_OK;
}

tq_status tq_bs_contract(const tq_bs *A, const tq_bs *B, int32_t n_legs, const int64_t *a_legs,
                         const int64_t *b_legs, const tq_contract_opts *opts, tq_stream stream,
                         tq_bs **out) {
  if (!out) return fail(TQ_ERR_INVALID, "out is NULL");
  tq_plan *P = nullptr;
  tq_bs *C = nullptr;
  TQ_CHECK(plan_build(A, B, n_legs, a_legs, b_legs, opts, (cudaStream_t)stream, &P, &C));
  tq_status st = plan_run(P, (cudaStream_t)stream);
  // the tensor-core kernel's bounded waits report through a device flag
  if (st == TQ_OK) st = plan_check(P, (cudaStream_t)stream);
  // the plan's scratch is released stream-ordered after the kernels that use it
  tq_plan_destroy(P);
  if (st != TQ_OK) {
    tq_bs_destroy(C);
    return st;
  }
  *out = C;
  return TQ_OK;
}

}  // extern "C"
