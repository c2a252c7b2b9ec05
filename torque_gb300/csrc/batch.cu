// Batches: many planned contractions as one numeric stage (one persistent
// tensor-core GEMM launch per wave of independent contractions), optionally
// captured once as a CUDA graph and replayed.
#include <memory>
#include <vector>

#include "ozaki.cuh"
#include "plan.cuh"

namespace tq {
tq_status plan_run(tq_plan *P, cudaStream_t s);
tq_status plan_check(tq_plan *P, cudaStream_t s);
}  // namespace tq

using namespace tq;

struct tq_batch {
  struct Wave {
    // the tensor-core plans of the wave: one launch per tile width in use
    std::vector<std::unique_ptr<OzBatchDev>> oz;
    std::vector<tq_plan *> hybrid;  // of those, plans with blocks grouped to plain FP64
    std::vector<tq_plan *> others;  // native-precision, rank-0 or empty plans
  };
  std::vector<std::unique_ptr<Wave>> waves;
  std::vector<tq_plan *> plans;
  std::vector<uint64_t> gens;  // each plan's schedule generation when the batch was built
  cudaStream_t capture_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t kernels = 0;
  ~tq_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (capture_stream) cudaStreamDestroy(capture_stream);
  }
};

// The batch's device tables point into its plans' schedule arrays, which a
// reschedule frees and rebuilds: such a batch must be built again.
static tq_status batch_current(const tq_batch *b) {
  for (size_t i = 0; i < b->plans.size(); i++)
    if (b->plans[i]->sched_gen != b->gens[i])
      return fail(TQ_ERR_INVALID,
                  "plan " + std::to_string(i) +
                      " was rescheduled after the batch was built; build the batch again");
  return TQ_OK;
}

static void batch_drop_graph(tq_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

static tq_status batch_run(tq_batch *b, cudaStream_t s) {
  for (auto &w : b->waves) {
    for (auto &oz : w->oz) {
      {
        NvtxRange r("tq_prepare");
        TQ_CHECK(oz_batch_prepare(*oz, s));
      }
      NvtxRange r("tq_gemm");
      TQ_CHECK(oz_batch_gemm(*oz, s));
    }
    for (tq_plan *P : w->hybrid) {
      NvtxRange r("tq_gemm_native");
      TQ_CHECK(run_hybrid_native(P, s));
    }
    for (tq_plan *P : w->others) TQ_CHECK(plan_run(P, s));
  }
  return TQ_OK;
}

extern "C" {

tq_status tq_batch_create(tq_plan *const *plans, int32_t n, const int32_t *wave, tq_stream stream,
                          tq_batch **out) {
  if (!out || (n > 0 && !plans)) return fail(TQ_ERR_INVALID, "NULL argument");
  if (n < 0) return fail(TQ_ERR_INVALID, "negative plan count");
  for (int32_t i = 0; i < n; i++) {
    if (!plans[i]) return fail(TQ_ERR_INVALID, "plan is NULL");
    if (!plans[i]->sched_ok) return fail(TQ_ERR_INVALID, "a plan's last reschedule failed");
    if (wave && i && wave[i] < wave[i - 1])
      return fail(TQ_ERR_INVALID, "waves must be non-decreasing");
  }
  cudaStream_t s = (cudaStream_t)stream;
  std::unique_ptr<tq_batch> b(new tq_batch());
  b->plans.assign(plans, plans + n);
  for (int32_t k = 0; k < n; k++) b->gens.push_back(plans[k]->sched_gen);
  int32_t i = 0;
  while (i < n) {
    const int32_t wv = wave ? wave[i] : 0;
    std::unique_ptr<tq_batch::Wave> w(new tq_batch::Wave());
    std::vector<OzJob> jobs[3];
    std::vector<OzSide> sides[3];
    for (; i < n && (wave ? wave[i] : 0) == wv; i++) {
      tq_plan *P = plans[i];
      if (P->tc && P->C->rank > 0 && P->tc_tiles > 0) {
        const int k = P->tile_n == 32 ? 0 : P->tile_n == 64 ? 1 : 2;
        jobs[k].push_back(P->tc_job);
        sides[k].push_back(P->tc_side[0]);
        sides[k].push_back(P->tc_side[1]);
        if (P->hyb_tiles) w->hybrid.push_back(P);
      } else {
        w->others.push_back(P);
      }
    }
    for (int k = 0; k < 3; k++) {
      if (jobs[k].empty()) continue;
      std::unique_ptr<OzBatchDev> oz(new OzBatchDev());
      TQ_CHECK(oz_batch_build(jobs[k], sides[k], s, *oz));
      w->oz.push_back(std::move(oz));
    }
    b->waves.push_back(std::move(w));
  }
  *out = b.release();
  return TQ_OK;
}

tq_status tq_batch_execute(tq_batch *b, tq_stream stream) {
  if (!b) return fail(TQ_ERR_INVALID, "batch is NULL");
  TQ_CHECK(batch_current(b));
  const int64_t k0 = tq_debug_kernel_launches();
  TQ_CHECK(batch_run(b, (cudaStream_t)stream));
  b->kernels = tq_debug_kernel_launches() - k0;
  return TQ_OK;
}

tq_status tq_batch_graph_launch(tq_batch *b, tq_stream stream) {
  if (!b) return fail(TQ_ERR_INVALID, "batch is NULL");
  TQ_CHECK(batch_current(b));
  if (!b->exec) {
    // capture on a private stream (the legacy stream cannot be captured), made
    // once per batch; a failed capture or instantiation leaves no graph behind
    if (!b->capture_stream)
      TQ_CUDA(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking));
    batch_drop_graph(b);
    TQ_CUDA(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal));
    const int64_t k0 = tq_debug_kernel_launches();
    tq_status st = batch_run(b, b->capture_stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
    if (st != TQ_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (st != TQ_OK) return st;
      TQ_CUDA(e);
    }
    b->graph = g;
    b->kernels = tq_debug_kernel_launches() - k0;
    const cudaError_t ei = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (ei != cudaSuccess) {
      b->exec = nullptr;
      batch_drop_graph(b);
      TQ_CUDA(ei);
    }
  }
  TQ_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  return TQ_OK;
}

tq_status tq_batch_check(tq_batch *b, tq_stream stream) {
  if (!b) return fail(TQ_ERR_INVALID, "batch is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CUDA(cudaStreamSynchronize(s));
  for (auto &w : b->waves) {
    for (auto &oz : w->oz) TQ_CHECK(oz_batch_check(*oz, s));
    for (tq_plan *P : w->others) TQ_CHECK(plan_check(P, s));
  }
  return TQ_OK;
}

tq_status tq_batch_kernels(const tq_batch *b, int64_t *kernels) {
  if (!b || !kernels) return fail(TQ_ERR_INVALID, "NULL argument");
  *kernels = b->kernels;
  return TQ_OK;
}

tq_status tq_batch_destroy(tq_batch *b) {
  delete b;
  return TQ_OK;
}

}  // extern "C"
