// Schedule autotuning: the exhaustive tuner (every candidate schedule run and
// timed on the device, its error measured against the plain FP64 result) and
// the contraction features the learned cost model reads.
//
// A schedule is a tq_contract_opts: precision and slice count, tensor-core tile
// width, and block grouping (the fill threshold below which an output block runs
// in plain FP64).  The tuner reuses one plan's symbolic stage for every
// candidate (tq_plan_reschedule), so a candidate costs its numeric stage only.
#include <cmath>
#include <cstring>
#include <vector>

#include "gemm.cuh"
#include "plan.cuh"

namespace tq {

// max |x - y| and max |y| over n doubles (non-negative doubles order like their
// bit patterns, so the maxima are integer atomics).
__global__ void maxdiff_kernel(const double *x, const double *y, int64_t n,
                               unsigned long long *out) {
  __shared__ unsigned long long rd[256], rr[256];
  unsigned long long md = 0, mr = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long d = (unsigned long long)__double_as_longlong(fabs(x[i] - y[i]));
    const unsigned long long r = (unsigned long long)__double_as_longlong(fabs(y[i]));
    md = d > md ? d : md;
    mr = r > mr ? r : mr;
  }
  rd[threadIdx.x] = md;
  rr[threadIdx.x] = mr;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      rd[threadIdx.x] = rd[threadIdx.x] > rd[threadIdx.x + w] ? rd[threadIdx.x] : rd[threadIdx.x + w];
      rr[threadIdx.x] = rr[threadIdx.x] > rr[threadIdx.x + w] ? rr[threadIdx.x] : rr[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicMax(&out[0], rd[0]);
    atomicMax(&out[1], rr[0]);
  }
}

// flop-weighted histograms of the block GEMM sizes m, n, k over all pairs:
// bin 0 for sizes below 8, then one bin per octave up to 512 and above.
__device__ __forceinline__ int size_bin(int64_t x) {
  if (x < 8) return 0;
  const int l = 63 - __clzll((long long)x) - 2;
  return l > 7 ? 7 : l;
}

__global__ void feature_kernel(DevBS A, DevBS B, LegSpec L, const int32_t *pa, const int32_t *pb,
                               int64_t n_pairs, double *bins) {
  __shared__ double h[24];
  if (threadIdx.x < 24) h[threadIdx.x] = 0.0;
  __syncthreads();
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n_pairs) {
    const int64_t i = pa[p], j = pb[p];
    int64_t m = 1, n = 1, k = 1;
    for (int q = 0; q < L.nfa; q++)
      m *= A.end[i * A.rank + L.fa[q]] - A.begin[i * A.rank + L.fa[q]] + 1;
    for (int q = 0; q < L.nfb; q++)
      n *= B.end[j * B.rank + L.fb[q]] - B.begin[j * B.rank + L.fb[q]] + 1;
    int64_t cb[TQ_MAXR], ce[TQ_MAXR];
    contraction_range(A, B, L, i, j, cb, ce);
    for (int c = 0; c < L.nc; c++) k *= ce[c] - cb[c] + 1;
    const double w = 2.0 * (double)m * (double)n * (double)k;
    atomicAdd(&h[size_bin(m)], w);
    atomicAdd(&h[8 + size_bin(n)], w);
    atomicAdd(&h[16 + size_bin(k)], w);
  }
  __syncthreads();
  if (threadIdx.x < 24 && h[threadIdx.x] != 0.0) atomicAdd(&bins[threadIdx.x], h[threadIdx.x]);
}

static tq_status plan_features(const tq_plan *P, double target, float *f, cudaStream_t s) {
  std::memset(f, 0, TQ_N_FEATURES * sizeof(float));
  const LegSpec &L = P->L;
  double cdim = 1.0;
  for (int c = 0; c < L.nc; c++) cdim *= (double)P->A->dimension[L.al[c]];
  f[0] = (float)(-std::log10(target > 0 ? target : 1e-300) / 16.0);
  f[1] = (float)(P->A->rank / 8.0);
  f[2] = (float)(P->B->rank / 8.0);
  f[3] = (float)(L.nc / 4.0);
  f[4] = (float)(std::log2(cdim) / 32.0);
  f[5] = (float)(std::log2(P->flops + 1.0) / 48.0);
  f[6] = (float)(std::log2((double)P->n_pairs + 1.0) / 24.0);
  f[7] = (float)(std::log2((double)P->n_out + 1.0) / 24.0);
  if (P->n_pairs == 0) return TQ_OK;
  DevArray<double> bins;
  TQ_CHECK(bins.alloc(24, s));
  TQ_CUDA(cudaMemsetAsync(bins.p, 0, 24 * 8, s));
  count_launch(), feature_kernel<<<(unsigned)((P->n_pairs + 255) / 256), 256, 0, s>>>(
      P->A->view(), P->B->view(), L, P->pa.p, P->pb.p, P->n_pairs, bins.p);
  TQ_CUDA(cudaGetLastError());
  double h[24];
  TQ_CUDA(cudaMemcpyAsync(h, bins.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  for (int g = 0; g < 3; g++) {
    double tot = 0.0;
    for (int b = 0; b < 8; b++) tot += h[8 * g + b];
    for (int b = 0; b < 8; b++) f[8 + 8 * g + b] = tot > 0 ? (float)(h[8 * g + b] / tot) : 0.f;
  }
  return TQ_OK;
}

// The numeric stage of P once, with events around it; ms = elapsed time.
static tq_status timed_run(tq_plan *P, cudaEvent_t e0, cudaEvent_t e1, cudaStream_t s, float *ms) {
  TQ_CUDA(cudaEventRecord(e0, s));
  TQ_CHECK(plan_run(P, s));
  TQ_CUDA(cudaEventRecord(e1, s));
  TQ_CHECK(plan_check(P, s));
  TQ_CUDA(cudaEventSynchronize(e1));
  TQ_CUDA(cudaEventElapsedTime(ms, e0, e1));
  return TQ_OK;
}

struct EventPair {
  cudaEvent_t e[2] = {nullptr, nullptr};
  ~EventPair() {
    for (auto x : e)
      if (x) cudaEventDestroy(x);
  }
};

}  // namespace tq

using namespace tq;

extern "C" {

tq_status tq_plan_features(const tq_plan *plan, double target_rel_err, float *features,
                           tq_stream stream) {
  if (!plan || !features) return fail(TQ_ERR_INVALID, "NULL argument");
  return plan_features(plan, target_rel_err, features, (cudaStream_t)stream);
}

}  // extern "C"

namespace tq {
static tq_status autotune_run(tq_plan *plan, const tq_contract_opts &keep, double target_rel_err,
                              tq_tune_entry *cands, int32_t n_cands, int32_t reps, int32_t *best,
                              cudaStream_t s) {
  EventPair ev;
  TQ_CUDA(cudaEventCreate(&ev.e[0]));
  TQ_CUDA(cudaEventCreate(&ev.e[1]));
  // the plain FP64 result: the error reference of every candidate (timing
  // only, without it, when the target is negative)
  const bool measure = target_rel_err >= 0.0;
  const int64_t n = !measure ? 0 : plan->C->rank == 0 ? 1 : plan->C->n_elem;
  DevArray<double> ref;
  DevArray<unsigned long long> md;
  if (measure) {
    tq_contract_opts nat = keep;
    nat.precision = TQ_PREC_NATIVE;
    TQ_CHECK(plan_reschedule(plan, nat, s));
    TQ_CHECK(ref.alloc(std::max<int64_t>(n, 1), s));
    TQ_CHECK(md.alloc(2, s));
    TQ_CHECK(plan_run(plan, s));
    if (n) TQ_CUDA(cudaMemcpyAsync(ref.p, plan->C->data, n * 8, cudaMemcpyDeviceToDevice, s));
  }
  *best = -1;
  float best_ms = 0.f;
  for (int32_t c = 0; c < n_cands; c++) {
    tq_tune_entry &E = cands[c];
    E.opts.layout = keep.layout;
    E.ms = 0.f;
    E.rel_err = 0.0;
    E.status = plan_reschedule(plan, E.opts, s);
    if (E.status != TQ_OK) continue;
    float ms = 0.f, mn = 0.f;
    E.status = timed_run(plan, ev.e[0], ev.e[1], s, &ms);  // warm-up
    for (int32_t r = 0; r < reps && E.status == TQ_OK; r++) {
      E.status = timed_run(plan, ev.e[0], ev.e[1], s, &ms);
      mn = r == 0 || ms < mn ? ms : mn;
    }
    if (E.status != TQ_OK) continue;
    E.ms = mn;
    unsigned long long h[2] = {0, 0};
    if (n) {
      TQ_CUDA(cudaMemsetAsync(md.p, 0, 16, s));
      const int64_t g = std::min<int64_t>((n + 255) / 256, 4096);
      count_launch(), maxdiff_kernel<<<(unsigned)g, 256, 0, s>>>((const double *)plan->C->data,
                                                                 ref.p, n, md.p);
      TQ_CUDA(cudaGetLastError());
      TQ_CUDA(cudaMemcpyAsync(h, md.p, 16, cudaMemcpyDeviceToHost, s));
      TQ_CUDA(cudaStreamSynchronize(s));
    }
    double dmax, rmax;
    std::memcpy(&dmax, &h[0], 8);
    std::memcpy(&rmax, &h[1], 8);
    E.rel_err = !measure ? -1.0 : rmax > 0 ? dmax / rmax : (dmax > 0 ? INFINITY : 0.0);
    if ((!measure || E.rel_err <= target_rel_err) && (*best < 0 || E.ms < best_ms)) {
      *best = c;
      best_ms = E.ms;
    }
  }
  // leave the plan with its own schedule, or the winner's
  const tq_contract_opts fin = *best >= 0 ? cands[*best].opts : keep;
  TQ_CHECK(plan_reschedule(plan, fin, s));
  return TQ_OK;
}
}  // namespace tq

extern "C" {

tq_status tq_autotune(tq_plan *plan, double target_rel_err, tq_tune_entry *cands,
                      int32_t n_cands, int32_t reps, int32_t *best, tq_stream stream) {
  if (!plan || (n_cands > 0 && !cands) || !best) return fail(TQ_ERR_INVALID, "NULL argument");
  if (n_cands < 0 || reps < 1) return fail(TQ_ERR_INVALID, "bad candidate or repetition count");
  if (plan->A->dtype != TQ_F64) return fail(TQ_ERR_UNSUPPORTED, "the tuner takes float64 tensors");
  cudaStream_t s = (cudaStream_t)stream;
  const tq_contract_opts keep = plan->opts;
  const tq_status st = autotune_run(plan, keep, target_rel_err, cands, n_cands, reps, best, s);
  if (st != TQ_OK) {
    // every failure leaves the plan on the caller's schedule (the first error's
    // message is kept)
    const std::string msg = tq_last_error_string();
    *best = -1;
    if (plan_reschedule(plan, keep, s) == TQ_OK) fail(st, msg);
  }
  return st;
}

}  // extern "C"
