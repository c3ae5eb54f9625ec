// C ABI of libfastjet_gb300.so (declarations: include/fastjet_gb300.h).
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include <cuda_runtime.h>

#include "fastjet_gb300.h"
#include "fjg_context.h"

static_assert(fjg::kLargeMaxN == FJG_MAX_EVENT_PARTICLES, "the C ABI states the kernels' size limit");

using fjg::BatchArgs;

namespace {
thread_local std::string g_thread_error;
}  // namespace

void fjg::set_thread_error(const char* msg) { g_thread_error = msg; }

namespace fjg {

fjg_status set_error(fjg_ctx* ctx, fjg_status st, const std::string& msg) {
  if (ctx)
    ctx->last_error = msg;
  else
    g_thread_error = msg;
  return st;
}

fjg_status cuda_error(fjg_ctx* ctx, cudaError_t err, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(err) + ": " + cudaGetErrorString(err);
  return set_error(ctx, err == cudaErrorMemoryAllocation ? FJG_ENOMEM : FJG_ECUDA, m);
}

fjg_status status_to_error(fjg_ctx* ctx, int st) {
  if (!st) return FJG_OK;
  if (st & kStatusTooBig) return set_error(ctx, FJG_ETOOBIG, "an event exceeds the supported particle count");
  if (st & kStatusInternal)
    return set_error(ctx, FJG_EKERNEL, "a clustering kernel found no candidate (non-finite input?)");
  return set_error(ctx, FJG_EINVAL, "an event has a non-finite momentum component, or the event offsets are invalid");
}

bool valid_algo(int a) { return a == FJG_KT || a == FJG_CAM || a == FJG_ANTIKT; }

cudaError_t ScratchSet::reserve_lists(int n_events) {
  if (n_events < 1) n_events = 1;
  if (sc.order && sc.cap_events >= n_events) return cudaSuccess;
  int cap = n_events + n_events / 4 + 64;
  const size_t hist_bytes = (sizeof(int32_t) * kHistBins + 255) & ~size_t(255);
  size_t bytes = sizeof(int32_t) * (size_t)kNumQueues * cap + 256 + hist_bytes;
  cudaError_t err = lists.reserve(bytes);
  if (err != cudaSuccess) return err;
  char* p = static_cast<char*>(lists.ptr);
  sc.offsets1 = reinterpret_cast<int64_t*>(p);
  sc.counts = reinterpret_cast<int32_t*>(p + 64);
  sc.queues = reinterpret_cast<int*>(p + 128);
  sc.status = reinterpret_cast<int*>(p + 192);
  sc.hist = reinterpret_cast<int32_t*>(p + 256);
  sc.order = reinterpret_cast<int32_t*>(p + 256 + hist_bytes);
  sc.cap_events = cap;
  err = cudaMemset(sc.status, 0, sizeof(int));
  if (err == cudaSuccess) err = cudaDeviceSynchronize();
  return err;
}

cudaError_t ScratchSet::reserve_ws(int64_t particles) {
  if (particles < 1) particles = 1;
  if (sc.ws && sc.ws_stride >= particles) return cudaSuccess;
  const int64_t stride = particles + particles / 4 + 1024;
  cudaError_t err = ws.reserve(sizeof(double) * kWsFields * (size_t)stride);
  if (err != cudaSuccess) return err;
  sc.ws = static_cast<double*>(ws.ptr);
  sc.ws_stride = (int64_t)(ws.cap / (sizeof(double) * kWsFields));
  return cudaSuccess;
}

cudaError_t ScratchSet::reserve_large(int64_t particles) {
  if (particles <= kSmemMaxN) return cudaSuccess;
  if (sc.large_ws && sc.large_ws_particles >= particles) return cudaSuccess;
  cudaError_t err = large.reserve((size_t)kLargeWsBytesPerParticle * (size_t)particles + 256);
  if (err != cudaSuccess) return err;
  sc.large_ws = static_cast<unsigned char*>(large.ptr);
  sc.large_ws_particles = (int64_t)((large.cap - 256) / kLargeWsBytesPerParticle);
  return cudaSuccess;
}

}  // namespace fjg

using fjg::cuda_error;
using fjg::DeviceGuard;
using fjg::set_error;
using fjg::valid_algo;

namespace {

// Read and clear the kernels' status word (synchronises the stream).
fjg_status take_status(fjg_ctx* ctx, cudaStream_t s) {
  int st = 0;
  cudaError_t err = cudaMemcpyAsync(&st, ctx->scratch.sc.status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return cuda_error(ctx, err, "clustering");
  if (st) {
    cudaMemsetAsync(ctx->scratch.sc.status, 0, sizeof(int), s);
    cudaStreamSynchronize(s);
  }
  return fjg::status_to_error(ctx, st);
}

}  // namespace

extern "C" {

const char* fjg_status_string(fjg_status s) {
  switch (s) {
    case FJG_OK: return "ok";
    case FJG_EINVAL: return "invalid argument";
    case FJG_ENOMEM: return "out of memory";
    case FJG_ECUDA: return "CUDA error";
    case FJG_ETOOBIG: return "event too large";
    case FJG_ETIMEDOUT: return "timed out";
    case FJG_EAGAIN: return "try again";
    case FJG_EKERNEL: return "kernel error";
  }
  return "unknown status";
}

const char* fjg_last_error(const fjg_ctx* ctx) { return ctx ? ctx->last_error.c_str() : g_thread_error.c_str(); }

fjg_status fjg_ctx_create(int device, fjg_ctx** out) {
  if (!out) return set_error(nullptr, FJG_EINVAL, "out is null");
  *out = nullptr;
  int count = 0;
  cudaError_t err = cudaGetDeviceCount(&count);
  if (err != cudaSuccess) return cuda_error(nullptr, err, "cudaGetDeviceCount");
  if (device < 0 || device >= count) return set_error(nullptr, FJG_EINVAL, "no such CUDA device");
  fjg_ctx* ctx = new (std::nothrow) fjg_ctx();
  if (!ctx) return set_error(nullptr, FJG_ENOMEM, "host allocation failed");
  ctx->device = device;
  DeviceGuard g(device);
  err = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  for (int b = 0; b < fjg::kNumQueues && err == cudaSuccess; ++b) {
    err = cudaStreamCreateWithFlags(&ctx->side[b], cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&ctx->ev_join[b], cudaEventDisableTiming);
  }
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
  if (err == cudaSuccess) err = ctx->scratch.reserve_lists(1024);
#ifdef FJG_PHASE_CLOCKS
  if (err == cudaSuccess) err = cudaMalloc(&ctx->phase, sizeof(unsigned long long) * fjg::kPhSlots);
  if (err == cudaSuccess) err = cudaMemset(ctx->phase, 0, sizeof(unsigned long long) * fjg::kPhSlots);
#endif
  if (err != cudaSuccess) {
    fjg_status st = cuda_error(nullptr, err, "context creation");
    fjg_ctx_destroy(ctx);
    return st;
  }
  *out = ctx;
  return FJG_OK;
}

void fjg_ctx_destroy(fjg_ctx* ctx) {
  if (!ctx) return;
  DeviceGuard g(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (int b = 0; b < fjg::kNumQueues; ++b) {
    if (ctx->side[b]) {
      cudaStreamSynchronize(ctx->side[b]);
      cudaStreamDestroy(ctx->side[b]);
    }
    if (ctx->ev_join[b]) cudaEventDestroy(ctx->ev_join[b]);
  }
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->phase) cudaFree(ctx->phase);
  ctx->scratch.release();
  ctx->io.release();
  ctx->single.release();
  ctx->select_scratch.release();
  delete ctx;
}

void* fjg_ctx_stream(fjg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

fjg_status fjg_phase_clocks(fjg_ctx* ctx, unsigned long long* out, int n, int reset) {
  if (!ctx || (!out && n > 0)) return set_error(ctx, FJG_EINVAL, "null argument");
  if (!ctx->phase) return set_error(ctx, FJG_EINVAL, "library built without FJG_PHASE_CLOCKS");
  DeviceGuard g(ctx->device);
  unsigned long long buf[fjg::kPhSlots];
  cudaError_t err = cudaStreamSynchronize(ctx->stream);
  if (err == cudaSuccess) err = cudaMemcpy(buf, ctx->phase, sizeof(buf), cudaMemcpyDeviceToHost);
  if (err == cudaSuccess && reset) err = cudaMemset(ctx->phase, 0, sizeof(buf));
  if (err != cudaSuccess) return cuda_error(ctx, err, "phase counters");
  for (int k = 0; k < n && k < fjg::kPhSlots; ++k) out[k] = buf[k];
  return FJG_OK;
}

fjg_status fjg_ctx_check(fjg_ctx* ctx) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  DeviceGuard g(ctx->device);
  for (int b = 0; b < fjg::kNumQueues; ++b) cudaStreamSynchronize(ctx->side[b]);
  return take_status(ctx, ctx->stream);
}

fjg_status fjg_cluster_batch(fjg_ctx* ctx, const double* p4, const int64_t* offsets, int n_events, int64_t total,
                             const int32_t* algo, int algo_all, const double* radius, double r_all,
                             const fjg_outputs* out, void* stream) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (n_events < 0 || total < 0 || !offsets || !out || !out->n_jets) return set_error(ctx, FJG_EINVAL, "bad batch arguments");
  if (n_events == 0) return FJG_OK;
  if (total > 0 && (!p4 || !out->jets || !out->jet_label)) return set_error(ctx, FJG_EINVAL, "null buffer");
  if (!algo && !valid_algo(algo_all)) return set_error(ctx, FJG_EINVAL, "bad algorithm");
  if (!radius && !fjg::valid_radius(r_all)) return set_error(ctx, FJG_EINVAL, "R must be finite and >= 0");
  DeviceGuard g(ctx->device);
  cudaError_t err = ctx->scratch.reserve_lists(n_events);
  if (err == cudaSuccess) err = ctx->scratch.reserve_ws(total);
  if (err == cudaSuccess) err = ctx->scratch.reserve_large(total);
  if (err != cudaSuccess) return cuda_error(ctx, err, "scratch allocation");
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  BatchArgs A{};
  A.phase = ctx->phase;
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
  A.status = ctx->scratch.sc.status;
  err = fjg::launch_batch(A, ctx->scratch.sc, n_events, ctx->num_sms, ctx->tune, s, ctx->side, &ctx->ev_fork,
                          ctx->ev_join);
  if (err != cudaSuccess) return cuda_error(ctx, err, "batch launch");
  return FJG_OK;
}

fjg_status fjg_cluster_batch_host(fjg_ctx* ctx, const double* p4, const int64_t* offsets, int n_events,
                                  const int32_t* algo, int algo_all, const double* radius, double r_all,
                                  const fjg_outputs* out) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (n_events < 0 || !offsets || !out || !out->n_jets) return set_error(ctx, FJG_EINVAL, "bad batch arguments");
  if (n_events == 0) return FJG_OK;
  const int64_t total = offsets[n_events];
  if (offsets[0] != 0 || total < 0) return set_error(ctx, FJG_EINVAL, "offsets must start at 0");
  for (int e = 0; e < n_events; ++e)
    if (offsets[e + 1] < offsets[e]) return set_error(ctx, FJG_EINVAL, "offsets must be non-decreasing");
  if (total > 0 && (!p4 || !out->jets || !out->jet_label)) return set_error(ctx, FJG_EINVAL, "null buffer");
  DeviceGuard g(ctx->device);
  // device layout: p4 | offsets | algo | radius | jets | labels | n_jets | history | owner
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t b_p4 = al(sizeof(double) * 4 * total), b_off = al(sizeof(int64_t) * (n_events + 1));
  const size_t b_algo = algo ? al(sizeof(int32_t) * n_events) : 0, b_rad = radius ? al(sizeof(double) * n_events) : 0;
  const size_t b_jets = al(sizeof(double) * 4 * total), b_lab = al(sizeof(int32_t) * total);
  const size_t b_nj = al(sizeof(int32_t) * n_events);
  const size_t b_hist = out->history ? al(sizeof(fjg_step) * total) : 0;
  const size_t b_own = out->owner ? al(sizeof(int32_t) * total) : 0;
  cudaError_t err = ctx->io.reserve(b_p4 + b_off + b_algo + b_rad + b_jets + b_lab + b_nj + b_hist + b_own);
  if (err != cudaSuccess) return cuda_error(ctx, err, "device buffers");
  char* d = static_cast<char*>(ctx->io.ptr);
  double* d_p4 = reinterpret_cast<double*>(d);
  d += b_p4;
  int64_t* d_off = reinterpret_cast<int64_t*>(d);
  d += b_off;
  int32_t* d_algo = algo ? reinterpret_cast<int32_t*>(d) : nullptr;
  d += b_algo;
  double* d_rad = radius ? reinterpret_cast<double*>(d) : nullptr;
  d += b_rad;
  fjg_outputs dout{};
  dout.jets = reinterpret_cast<double*>(d);
  d += b_jets;
  dout.jet_label = reinterpret_cast<int32_t*>(d);
  d += b_lab;
  dout.n_jets = reinterpret_cast<int32_t*>(d);
  d += b_nj;
  dout.history = out->history ? reinterpret_cast<fjg_step*>(d) : nullptr;
  d += b_hist;
  dout.owner = out->owner ? reinterpret_cast<int32_t*>(d) : nullptr;
  cudaStream_t s = ctx->stream;
  err = cudaMemcpyAsync(d_p4, p4, sizeof(double) * 4 * total, cudaMemcpyHostToDevice, s);
  if (err == cudaSuccess) err = cudaMemcpyAsync(d_off, offsets, sizeof(int64_t) * (n_events + 1), cudaMemcpyHostToDevice, s);
  if (err == cudaSuccess && algo) err = cudaMemcpyAsync(d_algo, algo, sizeof(int32_t) * n_events, cudaMemcpyHostToDevice, s);
  if (err == cudaSuccess && radius) err = cudaMemcpyAsync(d_rad, radius, sizeof(double) * n_events, cudaMemcpyHostToDevice, s);
  if (err != cudaSuccess) return cuda_error(ctx, err, "input copy");
  fjg_status st = fjg_cluster_batch(ctx, d_p4, d_off, n_events, total, d_algo, algo_all, d_rad, r_all, &dout, s);
  if (st != FJG_OK) return st;
  err = cudaMemcpyAsync(out->n_jets, dout.n_jets, sizeof(int32_t) * n_events, cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaMemcpyAsync(out->jets, dout.jets, sizeof(double) * 4 * total, cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaMemcpyAsync(out->jet_label, dout.jet_label, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess && out->history)
    err = cudaMemcpyAsync(out->history, dout.history, sizeof(fjg_step) * total, cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess && out->owner)
    err = cudaMemcpyAsync(out->owner, dout.owner, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, s);
  if (err != cudaSuccess) return cuda_error(ctx, err, "output copy");
  return take_status(ctx, s);
}

fjg_status fjg_cluster_event(fjg_ctx* ctx, const double* p4, int n, int algo, double r, double* jets,
                             int32_t* jet_label, int32_t* n_jets, fjg_step* history, int32_t* owner) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (n < 0 || !n_jets || (n > 0 && (!p4 || !jets || !jet_label))) return set_error(ctx, FJG_EINVAL, "bad arguments");
  if (!valid_algo(algo)) return set_error(ctx, FJG_EINVAL, "bad algorithm");
  if (!fjg::valid_radius(r)) return set_error(ctx, FJG_EINVAL, "R must be finite and >= 0");
  DeviceGuard g(ctx->device);
  cudaStream_t s = ctx->stream;
  if (n == 0) {
    cudaError_t err = cudaMemsetAsync(n_jets, 0, sizeof(int32_t), s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    return err == cudaSuccess ? FJG_OK : cuda_error(ctx, err, "fjg_cluster_event");
  }
  if (n > fjg::kLargeMaxN) return set_error(ctx, FJG_ETOOBIG, "event exceeds the supported particle count");
  cudaError_t werr = ctx->scratch.reserve_ws(n);
  if (werr == cudaSuccess) werr = ctx->scratch.reserve_large(n);
  if (werr != cudaSuccess) return cuda_error(ctx, werr, "workspace allocation");
  BatchArgs A{};
  A.phase = ctx->phase;
  A.p4 = p4;
  A.p4_stride = 4;
  A.algo = nullptr;
  A.radius = nullptr;
  A.algo_all = algo;
  A.r_all = r;
  A.jets = jets;
  A.jet_label = jet_label;
  A.n_jets = n_jets;
  A.history = reinterpret_cast<fjg::StepRec*>(history);
  A.owner = owner;
  A.status = ctx->scratch.sc.status;
  cudaError_t err = fjg::launch_single(A, ctx->scratch.sc, n, ctx->tune, s);
  if (err != cudaSuccess) return cuda_error(ctx, err, "fjg_cluster_event launch");
  return take_status(ctx, s);
}

fjg_status fjg_kinematics(fjg_ctx* ctx, const double* p4, int n, int algo, double* rap, double* phi, double* w,
                          void* stream) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (n < 0 || (n > 0 && (!p4 || !rap || !phi || !w))) return set_error(ctx, FJG_EINVAL, "bad arguments");
  if (!valid_algo(algo)) return set_error(ctx, FJG_EINVAL, "bad algorithm");
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  cudaError_t err = fjg::launch_kinematics(p4, n, algo, rap, phi, w, s);
  return err == cudaSuccess ? FJG_OK : cuda_error(ctx, err, "fjg_kinematics");
}

fjg_status fjg_cluster_pseudojets(fjg_ctx* ctx, fjg_pseudojet* particles, int size, int algo, double r,
                                  void* stream) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (size < 0 || (size > 0 && !particles)) return set_error(ctx, FJG_EINVAL, "bad arguments");
  if (!valid_algo(algo)) return set_error(ctx, FJG_EINVAL, "bad algorithm");
  if (!fjg::valid_radius(r)) return set_error(ctx, FJG_EINVAL, "R must be finite and >= 0");
  if (size == 0) return FJG_OK;
  if (size > fjg::kLargeMaxN) return set_error(ctx, FJG_ETOOBIG, "event exceeds the supported particle count");
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t b_jets = al(sizeof(double) * 4 * size), b_lab = al(sizeof(int32_t) * size);
  cudaError_t err = ctx->single.reserve(b_jets + b_lab + 256);
  if (err == cudaSuccess) err = ctx->scratch.reserve_ws(size);
  if (err == cudaSuccess) err = ctx->scratch.reserve_large(size);
  if (err != cudaSuccess) return cuda_error(ctx, err, "device buffers");
  char* d = static_cast<char*>(ctx->single.ptr);
  double* jets = reinterpret_cast<double*>(d);
  int32_t* labels = reinterpret_cast<int32_t*>(d + b_jets);
  int32_t* nj = reinterpret_cast<int32_t*>(d + b_jets + b_lab);
  BatchArgs A{};
  // px of record s sits 8 bytes into the 40-byte record: a stride of 5 doubles
  A.p4 = reinterpret_cast<const double*>(reinterpret_cast<const char*>(particles) + 8);
  A.p4_stride = 5;
  A.algo_all = algo;
  A.r_all = r;
  A.jets = jets;
  A.jet_label = labels;
  A.n_jets = nj;
  A.status = ctx->scratch.sc.status;
  err = fjg::launch_single(A, ctx->scratch.sc, size, ctx->tune, s);
  if (err == cudaSuccess) err = fjg::launch_pseudojet_epilogue(particles, size, jets, labels, nj, s);
  if (err != cudaSuccess) return cuda_error(ctx, err, "fjg_cluster_pseudojets");
  return take_status(ctx, s);
}

}  // extern "C"
