// CUDA-graph capture of the batch path (fjg_graph_* in fastjet_gb300.h).
#include <new>

#include "fjg_context.h"

struct fjg_graph {
  fjg_ctx* ctx = nullptr;
  fjg::ScratchSet scratch;  // private: the graph's kernels keep these addresses
  cudaGraphExec_t exec = nullptr;
  cudaStream_t last = nullptr;
};

using fjg::cuda_error;
using fjg::DeviceGuard;
using fjg::set_error;

extern "C" {

fjg_status fjg_graph_capture_batch(fjg_ctx* ctx, const double* p4, const int64_t* offsets, int n_events,
                                   int64_t total, const int32_t* algo, int algo_all, const double* radius,
                                   double r_all, const fjg_outputs* out, fjg_graph** graph) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (!graph) return set_error(ctx, FJG_EINVAL, "graph is null");
  *graph = nullptr;
  if (n_events < 1 || total < 0 || !offsets || !out || !out->n_jets)
    return set_error(ctx, FJG_EINVAL, "bad batch arguments");
  if (total > 0 && (!p4 || !out->jets || !out->jet_label)) return set_error(ctx, FJG_EINVAL, "null buffer");
  if (!algo && !fjg::valid_algo(algo_all)) return set_error(ctx, FJG_EINVAL, "bad algorithm");
  if (!radius && !fjg::valid_radius(r_all)) return set_error(ctx, FJG_EINVAL, "R must be finite and >= 0");
  DeviceGuard dg(ctx->device);
  fjg_graph* g = new (std::nothrow) fjg_graph();
  if (!g) return set_error(ctx, FJG_ENOMEM, "host allocation failed");
  g->ctx = ctx;
  cudaError_t err = g->scratch.reserve_lists(n_events);
  if (err == cudaSuccess) err = g->scratch.reserve_ws(total);
  if (err == cudaSuccess) err = g->scratch.reserve_large(total);
  // resolve the per-device launch attributes and occupancies outside the capture
  for (int b = 0; b < fjg::kNumBuckets && err == cudaSuccess; ++b) fjg::variant_occupancy(ctx->tune.bucket[b].variant);
  if (err == cudaSuccess) err = fjg::configure_tiled();
  fjg::launch_priority(0);
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
  if (err != cudaSuccess) {
    fjg_graph_destroy(g);
    return cuda_error(ctx, err, "graph scratch");
  }
  fjg::BatchArgs A{};
  A.particles = total;
  A.p4 = p4;
  A.p4_stride = 4;
  A.offsets = offsets;
  A.algo = algo;
  A.radius = radius;
  A.algo_all = algo_all;
  A.r_all = r_all;
  A.jets = out->jets;
  A.jet_label = out->jet_label;
  A.n_jets = out->n_jets;
  A.history = reinterpret_cast<fjg::StepRec*>(out->history);
  A.owner = out->owner;
  A.status = g->scratch.sc.status;
  cudaGraph_t cg = nullptr;
  err = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (err == cudaSuccess) {
    cudaError_t lerr = fjg::launch_batch(A, g->scratch.sc, n_events, ctx->num_sms, ctx->tune, ctx->stream,
                                         ctx->side, &ctx->ev_fork, ctx->ev_join);
    err = cudaStreamEndCapture(ctx->stream, &cg);
    if (lerr != cudaSuccess) err = lerr;
  }
  if (err == cudaSuccess) err = cudaGraphInstantiate(&g->exec, cg, 0);
  if (cg) cudaGraphDestroy(cg);
  if (err != cudaSuccess) {
    cudaGetLastError();
    fjg_graph_destroy(g);
    return cuda_error(ctx, err, "graph capture");
  }
  g->last = ctx->stream;
  *graph = g;
  return FJG_OK;
}

fjg_status fjg_graph_launch(fjg_graph* g, void* stream) {
  if (!g || !g->exec) return set_error(nullptr, FJG_EINVAL, "graph is null");
  DeviceGuard dg(g->ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : g->ctx->stream;
  cudaError_t err = cudaGraphLaunch(g->exec, s);
  if (err != cudaSuccess) return cuda_error(g->ctx, err, "graph launch");
  g->last = s;
  return FJG_OK;
}

fjg_status fjg_graph_check(fjg_graph* g) {
  if (!g || !g->exec) return set_error(nullptr, FJG_EINVAL, "graph is null");
  DeviceGuard dg(g->ctx->device);
  int st = 0;
  cudaError_t err = cudaMemcpyAsync(&st, g->scratch.sc.status, sizeof(int), cudaMemcpyDeviceToHost, g->last);
  if (err == cudaSuccess) err = cudaStreamSynchronize(g->last);
  if (err != cudaSuccess) return cuda_error(g->ctx, err, "graph check");
  if (st) {
    cudaMemsetAsync(g->scratch.sc.status, 0, sizeof(int), g->last);
    cudaStreamSynchronize(g->last);
  }
  return fjg::status_to_error(g->ctx, st);
}

void fjg_graph_destroy(fjg_graph* g) {
  if (!g) return;
  DeviceGuard dg(g->ctx->device);
  if (g->last) cudaStreamSynchronize(g->last);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  g->scratch.release();
  delete g;
}

}  // extern "C"
