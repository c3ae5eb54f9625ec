// fjg_cluster_batch_noalloc: batched clustering that allocates nothing.
//
// Who needs it: callers that must not allocate device memory at the point of
// the call -- trigger or other real-time code that forbids allocation after
// initialisation (cudaMalloc/cudaFree can synchronise the device and take an
// unbounded time), or applications whose device memory is owned entirely by
// another allocator or capped by a quota.  Such callers also cannot create a
// library context, because fjg_ctx_create allocates the context's scratch.
//
// How: the bookkeeping the batch kernels need besides their inputs and outputs
// (per-list event lists, work-queue counters, the error word, the kernels'
// per-particle workspaces) lives in one
// file-scope device array of fixed size, kNoAllocScratchBytes, that every GPU
// which loads this library holds until the process exits.  The host cannot use
// the array's name as a device address, so the first call on each device
// looks the address up with cudaGetSymbolAddress (with that device current)
// and caches it.  Every call reads the kernels' status word back and
// synchronises its stream, so no call can be made inside stream capture.
// All calls share the array: each call clears the counters and the error word
// before its kernels run, and calls whose work overlaps on the GPU (different
// streams or host threads without ordering) race on it.
//
// Bounds: the input check refuses events whose range [offsets[e],
// offsets[e+1]) leaves [0, total) (total <= kNoAllocMaxParticles, the extent
// of the per-particle workspace) and reads no momentum past `total`.  An event above 4096 particles uses
// large_ws_bytes(N) <= 93 N + 16 < kLargeWsBytesPerParticle * N bytes from
// kLargeWsBytesPerParticle * offsets[e] on, so its region ends inside the
// large workspace too (no margin is needed past the last particle).
#include <cstddef>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "fastjet_gb300.h"
#include "fjg_context.h"
#include "fjg_kernels.cuh"

namespace {

constexpr int kNoAllocMaxEvents = FJG_NOALLOC_MAX_EVENTS;
constexpr int kNoAllocMaxParticles = FJG_NOALLOC_MAX_PARTICLES;

struct NoAllocScratch {
  double ws[fjg::kWsFields * kNoAllocMaxParticles];    // exact per-particle state (overwritten per event)
  unsigned char large_ws[fjg::kLargeWsBytesPerParticle * kNoAllocMaxParticles];  // tiled-kernel state
  int32_t order[fjg::kNumQueues * kNoAllocMaxEvents];  // per-list event lists
  int32_t hist[fjg::kHistBins];                        // size histogram (zeroed per call)
  int32_t counts[fjg::kNumQueues];                     // events per list (zeroed per call)
  int32_t queues[fjg::kNumQueues];                     // work-queue heads (zeroed per call)
  int32_t status;                                      // kernel error bits (zeroed per call)
};

static_assert(sizeof(NoAllocScratch) <= FJG_NOALLOC_SCRATCH_BYTES, "scratch larger than documented");
static_assert(offsetof(NoAllocScratch, large_ws) % 16 == 0, "the tiled kernel reads 16 B records from large_ws");

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_setup_mu;
NoAllocScratch* g_scratch_addr[64] = {};  // device address per CUDA ordinal
int g_num_sms[64] = {};

fjg_status fail(fjg_status st, const char* msg) {
  fjg::set_thread_error(msg);
  return st;
}

}  // namespace

extern "C" fjg_status fjg_cluster_batch_noalloc(const double* p4, const int64_t* offsets, int n_events,
                                                int64_t total, const int32_t* algo, int algo_all,
                                                const double* radius, double r_all, const fjg_outputs* out,
                                                void* stream) {
  if (n_events < 0 || !offsets || !out || !out->n_jets) return fail(FJG_EINVAL, "bad batch arguments");
  if (n_events > kNoAllocMaxEvents)
    return fail(FJG_EINVAL, "fjg_cluster_batch_noalloc: more events than FJG_NOALLOC_MAX_EVENTS in one call");
  if (n_events == 0) return FJG_OK;
  if (!p4 || !out->jets || !out->jet_label) return fail(FJG_EINVAL, "null buffer");
  if (total < 0 || total > kNoAllocMaxParticles)
    return fail(FJG_EINVAL, "fjg_cluster_batch_noalloc: more particles than FJG_NOALLOC_MAX_PARTICLES in one call");
  if (!algo && !(algo_all == FJG_KT || algo_all == FJG_CAM || algo_all == FJG_ANTIKT))
    return fail(FJG_EINVAL, "bad algorithm");
  if (!radius && !fjg::valid_radius(r_all)) return fail(FJG_EINVAL, "R must be finite and >= 0");

  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(FJG_ECUDA, "no usable CUDA device");
  NoAllocScratch* sc_dev;
  int num_sms;
  {
    // set-up, once per device, with that device current
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
      void* ptr = nullptr;
      cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (err != cudaSuccess || !ptr) return fail(FJG_ECUDA, "cudaGetSymbolAddress of the static scratch failed");
      int sms = 0;
      err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (err != cudaSuccess || sms < 1) return fail(FJG_ECUDA, "cudaDeviceGetAttribute failed");
      g_num_sms[dev] = sms;
      g_scratch_addr[dev] = static_cast<NoAllocScratch*>(ptr);
    }
    sc_dev = g_scratch_addr[dev];
    num_sms = g_num_sms[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;

  fjg::Scratch sc{};
  sc.order = sc_dev->order;
  sc.counts = sc_dev->counts;
  sc.queues = sc_dev->queues;
  sc.status = &sc_dev->status;
  sc.offsets1 = nullptr;
  sc.cap_events = kNoAllocMaxEvents;
  sc.hist = sc_dev->hist;
  sc.ws = sc_dev->ws;
  sc.ws_stride = kNoAllocMaxParticles;
  sc.large_ws = sc_dev->large_ws;
  sc.large_ws_particles = kNoAllocMaxParticles;

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
  A.status = sc.status;

  // the array keeps the previous call's contents: clear the error word (the
  // launcher clears the bucket counters and queue heads)
  cudaError_t err = cudaMemsetAsync(sc.status, 0, sizeof(int32_t), s);
  if (err == cudaSuccess) err = fjg::launch_batch_on_stream(A, sc, n_events, num_sms, fjg::default_tuning(), s);
  int st = 0;
  if (err == cudaSuccess) err = cudaMemcpyAsync(&st, sc.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return fail(err == cudaErrorMemoryAllocation ? FJG_ENOMEM : FJG_ECUDA, cudaGetErrorString(err));
  // the same status words and messages as the context entry points
  return fjg::status_to_error(nullptr, st);
}
