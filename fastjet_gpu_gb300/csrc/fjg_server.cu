// Request server (fjg_server_* in fastjet_gb300.h): continuous batching of
// individually submitted events on one GPU.
//
// Memory.  An arena of `arena_particles` particle positions.  Each admitted
// event holds one contiguous range [start, start + n):
//   pinned, mapped host memory: the momenta's staging copy (written by the
//     host at admission), jets, jet labels, history and owner (written by the
//     kernels directly, read by the host on completion);
//   device memory: the momenta (copied from the staging range at admission,
//     on a copy stream that every launch waits for), the FP64 workspace
//     (kWsFields doubles per position) and the tiled kernel's workspace
//     (kLargeWsBytesPerParticle per position).  The particle and neighbour
//     state the kernels read is device-resident.
// A request also holds a completion slot: a flag in mapped host memory that
// its kernel raises (system-scope release store) once the event's outputs
// are written.
//
// Scheduling (on every submit and poll):
//   1. completions: raised flags are collected; a stream whose micro-batch is
//      complete (flags and its CUDA event) becomes idle again;
//   2. admission, first come first served: the head request gets an arena
//      range (first fit) and a slot, or everything waits;
//   3. launches: per size bucket (largest first), admitted requests go out as
//      one micro-batch on an idle stream, up to max_batch events and up to
//      the bucket's in-flight limit (its resident CTAs times oversubscribe).
// Micro-batches of different buckets and of the same bucket run concurrently
// on different streams, so requests that arrive while others are running
// start without waiting for them.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <unordered_map>
#include <vector>

#include "fjg_context.h"

using fjg::cuda_error;
using fjg::DeviceGuard;
using fjg::set_error;

namespace {

using Clock = std::chrono::steady_clock;

double micros(Clock::duration d) { return std::chrono::duration<double, std::micro>(d).count(); }

enum ReqState { kPending, kAdmitted, kRunning, kDone };

struct Req {
  uint64_t ticket = 0;
  int n = 0, algo = 0, bucket = 0;
  double r = 0.0;
  const double* src = nullptr;  // momenta until admission (owned copy or the caller's buffer)
  std::vector<double> copy;
  int64_t start = -1;
  int slot = -1;
  int state = kPending;
  int status = FJG_OK;
  int n_jets = 0;
  int64_t user = -1;  // replay: index of the event
  Clock::time_point t_submit, t_done;
};

// Per-stream descriptors of one micro-batch, in mapped host memory.
struct Block {
  int64_t* offsets;    // [2 max_batch] (start, end) pairs
  int32_t* algo;       // [max_batch]
  double* radius;      // [max_batch]
  int32_t* done_slot;  // [max_batch]
  int32_t* n_jets;     // [max_batch]
  int32_t* ev_status;  // [max_batch] per-event status bits (0: fine)
  int32_t* count;      // [1]
};

struct Lane {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  bool busy = false;
  int q = -1;  // queue of the micro-batch in flight
  std::vector<Req*> batch;
  Block host{}, dev{};
  int* d_queue = nullptr;   // work-queue head (device)
  int* d_status = nullptr;  // kernel status word (device)
  int* h_status = nullptr;  // its copy (pinned), valid once ev completes
  int attributed = 0;       // status bits of the micro-batch's requests seen so far
};

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct fjg_server {
  fjg_ctx* ctx = nullptr;
  fjg_server_config cfg{};
  // mapped host arena (host and device views)
  void* host_mem = nullptr;
  double *h_p4 = nullptr, *h_jets = nullptr, *d_jets = nullptr;
  double* d_p4dev = nullptr;       // device copy of the momenta (arena positions)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_copy = nullptr;   // after the last admission's copy
  int32_t *h_lab = nullptr, *d_lab = nullptr, *h_own = nullptr, *d_own = nullptr;
  fjg_step *h_hist = nullptr, *d_hist = nullptr;
  int32_t *h_done = nullptr, *d_done = nullptr;
  void* block_mem = nullptr;
  // device state
  void* dev_mem = nullptr;
  double* d_ws = nullptr;
  unsigned char* d_large = nullptr;
  int32_t* d_iota = nullptr;
  int* d_words = nullptr;
  int* h_words = nullptr;
  // bookkeeping
  std::map<int64_t, int64_t> free_ranges;  // start -> length
  std::vector<int> free_slots;
  std::deque<Req*> pending;
  std::deque<Req*> admitted[fjg::kNumQueues];
  std::deque<Req*> completed;
  std::unordered_map<uint64_t, Req*> returned;
  std::vector<Lane> lanes;
  int inflight[fjg::kNumQueues] = {};
  int limit[fjg::kNumQueues] = {};
  uint64_t next_ticket = 1;
  int outstanding = 0;  // submitted, not yet returned by poll
  int64_t launches = 0;  // clustering kernels launched (inputs are checked on the host at submission)
  bool failed = false;
};

namespace {

int queue_of(int n) {
  const int b = fjg::bucket_of(n);
  return b < 0 ? fjg::kLargeQueue : b;
}

int64_t arena_alloc(fjg_server* S, int64_t n) {
  for (auto it = S->free_ranges.begin(); it != S->free_ranges.end(); ++it) {
    if (it->second >= n) {
      const int64_t start = it->first, len = it->second;
      S->free_ranges.erase(it);
      if (len > n) S->free_ranges.emplace(start + n, len - n);
      return start;
    }
  }
  return -1;
}

void arena_free(fjg_server* S, int64_t start, int64_t n) {
  if (n <= 0) return;
  auto next = S->free_ranges.lower_bound(start);
  if (next != S->free_ranges.end() && start + n == next->first) {
    n += next->second;
    next = S->free_ranges.erase(next);
  }
  if (next != S->free_ranges.begin()) {
    auto prev = std::prev(next);
    if (prev->first + prev->second == start) {
      prev->second += n;
      return;
    }
  }
  S->free_ranges.emplace(start, n);
}

// A request's result status from its per-event status bits.
int event_status(int bits) {
  if (!bits) return FJG_OK;
  if (bits & fjg::kStatusTooBig) return FJG_ETOOBIG;
  if (bits & fjg::kStatusInternal) return FJG_EKERNEL;
  return FJG_EINVAL;
}

void finish(fjg_server* S, Req* r, int status) {
  r->status = status;
  r->state = kDone;
  r->t_done = Clock::now();
  S->completed.push_back(r);
}

cudaError_t launch_lane(fjg_server* S, Lane& L, int q, int m) {
  fjg_ctx* ctx = S->ctx;
  for (int i = 0; i < m; ++i) {
    Req* r = S->admitted[q].front();
    S->admitted[q].pop_front();
    L.host.offsets[2 * i] = r->start;
    L.host.offsets[2 * i + 1] = r->start + r->n;
    L.host.algo[i] = r->algo;
    L.host.radius[i] = r->r;
    L.host.done_slot[i] = r->slot;
    L.host.n_jets[i] = 0;
    L.host.ev_status[i] = 0;
    r->state = kRunning;
    L.batch.push_back(r);
  }
  *L.host.count = m;
  fjg::BatchArgs A{};
  A.p4 = S->d_p4dev;
  A.p4_stride = 4;
  A.offsets = L.dev.offsets;
  A.pairs = 1;
  A.algo = L.dev.algo;
  A.radius = L.dev.radius;
  A.order = S->d_iota;
  A.n_order = L.dev.count;
  A.queue = L.d_queue;
  A.ws = S->d_ws;
  A.ws_stride = S->cfg.arena_particles;
  A.jets = S->d_jets;
  A.jet_label = S->d_lab;
  A.n_jets = L.dev.n_jets;
  A.history = reinterpret_cast<fjg::StepRec*>(S->d_hist);
  A.owner = S->d_own;
  A.status = L.d_status;
  A.large_ws = S->d_large;
  A.tile_factor = ctx->tune.tile_factor;
  A.serve_order = 1;  // small events first: they are the latency-bound requests
  A.done = S->d_done;
  A.done_slot = L.dev.done_slot;
  A.ev_status = L.dev.ev_status;
  L.attributed = 0;
  // the momenta of the micro-batch were copied at admission
  cudaError_t err = cudaStreamWaitEvent(L.stream, S->ev_copy, 0);
  if (err == cudaSuccess) err = cudaMemsetAsync(L.d_queue, 0, 2 * sizeof(int), L.stream);  // queue head and status
  if (err != cudaSuccess) return err;
  if (S->cfg.flags & FJG_SERVE_DEVICE_CHECK) {
    // momenta checked on the device: a request with a non-finite component
    // gets its own status word set and is skipped by the clustering kernel
    err = fjg::launch_check_pairs(S->d_p4dev, L.dev.offsets, m, L.dev.ev_status, L.stream);
    if (err != cudaSuccess) return err;
  }
  if (q == fjg::kLargeQueue) {
    const int grid = std::min(m, ctx->num_sms * ctx->tune.large_ctas_per_sm);
    err = fjg::launch_tiled(A, grid, L.stream);
  } else {
    const int per_sm = fjg::bucket_per_sm(ctx->tune, q);
    err = fjg::launch_variant(ctx->tune.bucket[q].variant, A, std::min(m, ctx->num_sms * per_sm), per_sm, L.stream);
  }
  if (err == cudaSuccess) ++S->launches;
  if (err == cudaSuccess) err = cudaMemcpyAsync(L.h_status, L.d_status, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
  if (err == cudaSuccess) err = cudaEventRecord(L.ev, L.stream);
  L.busy = true;
  L.q = q;
  S->inflight[q] += m;
  return err;
}

// One pass of the scheduler; returns false after a CUDA error.
bool progress(fjg_server* S) {
  if (S->failed) return false;
  // 1. completions.  The event is queried before the flags are read: once it
  // has completed, every flag of its micro-batch must be up.
  for (Lane& L : S->lanes) {
    if (!L.busy) continue;
    const cudaError_t q = cudaEventQuery(L.ev);
    const bool ended = q != cudaErrorNotReady;
    const int st = (q == cudaSuccess) ? *L.h_status : (ended ? -1 : 0);
    for (size_t i = 0; i < L.batch.size(); ++i) {
      Req* r = L.batch[i];
      if (!r) continue;  // completed earlier (and possibly returned and released since)
      if (__atomic_load_n(&S->h_done[r->slot], __ATOMIC_ACQUIRE)) {
        r->n_jets = __atomic_load_n(&L.host.n_jets[i], __ATOMIC_ACQUIRE);
        const int bits = __atomic_load_n(&L.host.ev_status[i], __ATOMIC_ACQUIRE);
        L.attributed |= bits;
        S->inflight[r->bucket]--;
        finish(S, r, event_status(bits));  // a failed request fails alone
        L.batch[i] = nullptr;
      } else if (ended) {
        S->inflight[r->bucket]--;
        finish(S, r, q == cudaSuccess ? FJG_EKERNEL : FJG_ECUDA);
        L.batch[i] = nullptr;
      }
    }
    if (!ended) continue;
    // every status bit a clustering kernel raises is also recorded in the
    // event's own word and failed that request alone; a bit that no request
    // accounts for means the server can no longer be trusted
    if (st & ~L.attributed) S->failed = true;
    L.busy = false;
    L.batch.clear();
  }
  // 2. admission (first come, first served): the momenta go to the staging
  // range and are copied to the device arena on the copy stream
  bool copied = false;
  while (!S->pending.empty() && !S->free_slots.empty()) {
    Req* r = S->pending.front();
    const int64_t start = arena_alloc(S, r->n);
    if (start < 0) break;
    S->pending.pop_front();
    r->start = start;
    r->slot = S->free_slots.back();
    S->free_slots.pop_back();
    std::memcpy(S->h_p4 + 4 * start, r->src, sizeof(double) * 4 * (size_t)r->n);
    if (cudaMemcpyAsync(S->d_p4dev + 4 * start, S->h_p4 + 4 * start, sizeof(double) * 4 * (size_t)r->n,
                        cudaMemcpyHostToDevice, S->copy_stream) != cudaSuccess) {
      S->failed = true;
      return false;
    }
    copied = true;
    r->copy.clear();
    r->copy.shrink_to_fit();
    r->src = nullptr;
    __atomic_store_n(&S->h_done[r->slot], 0, __ATOMIC_RELEASE);
    r->state = kAdmitted;
    S->admitted[r->bucket].push_back(r);
  }
  if (copied && cudaEventRecord(S->ev_copy, S->copy_stream) != cudaSuccess) {
    S->failed = true;
    return false;
  }
  // 3. launches, smallest events first (they are the latency-bound
  // requests); events above 4096 particles take at most half of the streams
  // and of the SMs (a tiled-kernel CTA fills an SM's registers for the whole
  // event), so that they cannot hold every SM away from the small ones
  for (int q = 0; q <= fjg::kLargeQueue; ++q) {
    while (!S->admitted[q].empty() && S->inflight[q] < S->limit[q]) {
      Lane* idle = nullptr;
      int large_lanes = 0;
      for (Lane& L : S->lanes) {
        if (L.busy && L.q == fjg::kLargeQueue) ++large_lanes;
        if (!L.busy && !idle) idle = &L;
      }
      if (!idle) return true;
      if (q == fjg::kLargeQueue && 2 * large_lanes >= (int)S->lanes.size()) break;
      const int m = (int)std::min<int64_t>(
          {(int64_t)S->admitted[q].size(), (int64_t)S->cfg.max_batch, (int64_t)(S->limit[q] - S->inflight[q])});
      if (launch_lane(S, *idle, q, m) != cudaSuccess) {
        S->failed = true;
        return false;
      }
    }
  }
  return true;
}

void release_req(fjg_server* S, Req* r) {
  if (r->start >= 0) arena_free(S, r->start, r->n);
  if (r->slot >= 0) S->free_slots.push_back(r->slot);
  delete r;
}

fjg_status submit_req(fjg_server* S, Req* r) {
  r->ticket = S->next_ticket++;
  r->bucket = queue_of(r->n);
  if (!r->t_submit.time_since_epoch().count()) r->t_submit = Clock::now();
  S->outstanding++;
  if (r->n == 0) {
    r->src = nullptr;
    finish(S, r, FJG_OK);
    return FJG_OK;
  }
  S->pending.push_back(r);
  return FJG_OK;
}

fjg_status check_event(fjg_server* S, const double* p4, int n, int algo, double r) {
  if (n < 0 || (n > 0 && !p4)) return set_error(S->ctx, FJG_EINVAL, "bad event");
  if (!fjg::valid_algo(algo)) return set_error(S->ctx, FJG_EINVAL, "bad algorithm");
  if (!fjg::valid_radius(r)) return set_error(S->ctx, FJG_EINVAL, "R must be finite and >= 0");
  if (n > S->cfg.arena_particles || n > fjg::kLargeMaxN)
    return set_error(S->ctx, FJG_ETOOBIG, "event larger than the server's arena");
  if (!(S->cfg.flags & FJG_SERVE_DEVICE_CHECK))
    for (int64_t i = 0; i < 4 * (int64_t)n; ++i)
      if (!std::isfinite(p4[i])) return set_error(S->ctx, FJG_EINVAL, "non-finite momentum");
  return FJG_OK;
}

}  // namespace

extern "C" {

fjg_status fjg_server_create(fjg_ctx* ctx, const fjg_server_config* config, fjg_server** out) {
  if (!ctx || !out) return set_error(ctx, FJG_EINVAL, "null argument");
  *out = nullptr;
  fjg_server_config c{};
  if (config) c = *config;
  if (c.arena_particles <= 0) c.arena_particles = 1 << 22;
  if (c.max_inflight <= 0) c.max_inflight = 8192;
  if (c.streams <= 0) c.streams = 16;
  if (c.max_batch <= 0) c.max_batch = 512;
  if (c.oversubscribe <= 0) c.oversubscribe = 2;
  if (c.arena_particles > (int64_t)1 << 31 || c.streams > 256 || c.max_batch > 65536)
    return set_error(ctx, FJG_EINVAL, "server configuration out of range");
  DeviceGuard dg(ctx->device);
  fjg_server* S = new (std::nothrow) fjg_server();
  if (!S) return set_error(ctx, FJG_ENOMEM, "host allocation failed");
  S->ctx = ctx;
  S->cfg = c;
  const int64_t P = c.arena_particles;
  const bool hist = (c.flags & FJG_SERVE_HISTORY) != 0;
  const size_t b_p4 = al(32 * (size_t)P), b_jets = al(32 * (size_t)P), b_lab = al(4 * (size_t)P);
  const size_t b_hist = hist ? al(sizeof(fjg_step) * (size_t)P) : 0, b_own = hist ? al(4 * (size_t)P) : 0;
  const size_t b_done = al(4 * (size_t)c.max_inflight);
  const size_t per_block = al(16 * (size_t)c.max_batch) + al(4 * (size_t)c.max_batch) + al(8 * (size_t)c.max_batch) +
                           al(4 * (size_t)c.max_batch) + al(4 * (size_t)c.max_batch) + al(4 * (size_t)c.max_batch) +
                           256;
  cudaError_t err = cudaHostAlloc(&S->host_mem, b_p4 + b_jets + b_lab + b_hist + b_own + b_done,
                                  cudaHostAllocMapped | cudaHostAllocPortable);
  if (err == cudaSuccess)
    err = cudaHostAlloc(&S->block_mem, per_block * c.streams + al(8 * (size_t)c.streams),
                        cudaHostAllocMapped | cudaHostAllocPortable);
  const size_t b_ws = al(sizeof(double) * fjg::kWsFields * (size_t)P);
  const size_t b_large = al((size_t)fjg::kLargeWsBytesPerParticle * (size_t)P);
  const size_t b_iota = al(4 * (size_t)c.max_batch), b_words = al(8 * (size_t)c.streams);
  const size_t b_p4dev = al(32 * (size_t)P);
  if (err == cudaSuccess) err = cudaMalloc(&S->dev_mem, b_ws + b_large + b_iota + b_words + b_p4dev);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&S->copy_stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&S->ev_copy, cudaEventDisableTiming);
  auto dev_of = [&](void* h) {
    void* d = nullptr;
    if (err == cudaSuccess) err = cudaHostGetDevicePointer(&d, h, 0);
    return d;
  };
  if (err == cudaSuccess) {
    char* h = static_cast<char*>(S->host_mem);
    S->h_p4 = reinterpret_cast<double*>(h);
    S->h_jets = reinterpret_cast<double*>(h + b_p4);
    S->h_lab = reinterpret_cast<int32_t*>(h + b_p4 + b_jets);
    S->h_hist = hist ? reinterpret_cast<fjg_step*>(h + b_p4 + b_jets + b_lab) : nullptr;
    S->h_own = hist ? reinterpret_cast<int32_t*>(h + b_p4 + b_jets + b_lab + b_hist) : nullptr;
    S->h_done = reinterpret_cast<int32_t*>(h + b_p4 + b_jets + b_lab + b_hist + b_own);
    S->d_jets = static_cast<double*>(dev_of(S->h_jets));
    S->d_lab = static_cast<int32_t*>(dev_of(S->h_lab));
    S->d_hist = hist ? static_cast<fjg_step*>(dev_of(S->h_hist)) : nullptr;
    S->d_own = hist ? static_cast<int32_t*>(dev_of(S->h_own)) : nullptr;
    S->d_done = static_cast<int32_t*>(dev_of(S->h_done));
    char* d = static_cast<char*>(S->dev_mem);
    S->d_ws = reinterpret_cast<double*>(d);
    S->d_large = reinterpret_cast<unsigned char*>(d + b_ws);
    S->d_iota = reinterpret_cast<int32_t*>(d + b_ws + b_large);
    S->d_words = reinterpret_cast<int*>(d + b_ws + b_large + b_iota);
    S->d_p4dev = reinterpret_cast<double*>(d + b_ws + b_large + b_iota + b_words);
    std::memset(S->h_done, 0, 4 * (size_t)c.max_inflight);
  }
  std::vector<int32_t> iota(c.max_batch);
  for (int i = 0; i < c.max_batch; ++i) iota[i] = i;
  if (err == cudaSuccess) err = cudaMemcpy(S->d_iota, iota.data(), 4 * (size_t)c.max_batch, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    S->lanes.resize(c.streams);
    char* blk = static_cast<char*>(S->block_mem);
    S->h_words = reinterpret_cast<int*>(blk + per_block * c.streams);
    for (int k = 0; k < c.streams && err == cudaSuccess; ++k) {
      Lane& L = S->lanes[k];
      char* p = blk + per_block * k;
      L.host.offsets = reinterpret_cast<int64_t*>(p);
      p += al(16 * (size_t)c.max_batch);
      L.host.algo = reinterpret_cast<int32_t*>(p);
      p += al(4 * (size_t)c.max_batch);
      L.host.radius = reinterpret_cast<double*>(p);
      p += al(8 * (size_t)c.max_batch);
      L.host.done_slot = reinterpret_cast<int32_t*>(p);
      p += al(4 * (size_t)c.max_batch);
      L.host.n_jets = reinterpret_cast<int32_t*>(p);
      p += al(4 * (size_t)c.max_batch);
      L.host.ev_status = reinterpret_cast<int32_t*>(p);
      p += al(4 * (size_t)c.max_batch);
      L.host.count = reinterpret_cast<int32_t*>(p);
      L.dev.offsets = static_cast<int64_t*>(dev_of(L.host.offsets));
      L.dev.algo = static_cast<int32_t*>(dev_of(L.host.algo));
      L.dev.radius = static_cast<double*>(dev_of(L.host.radius));
      L.dev.done_slot = static_cast<int32_t*>(dev_of(L.host.done_slot));
      L.dev.n_jets = static_cast<int32_t*>(dev_of(L.host.n_jets));
      L.dev.ev_status = static_cast<int32_t*>(dev_of(L.host.ev_status));
      L.dev.count = static_cast<int32_t*>(dev_of(L.host.count));
      L.d_queue = S->d_words + 2 * k;
      L.d_status = S->d_words + 2 * k + 1;
      L.h_status = S->h_words + 2 * k + 1;
      if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
      if (err == cudaSuccess) err = cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming);
    }
  }
  if (err != cudaSuccess) {
    fjg_status st = cuda_error(ctx, err, "server creation");
    fjg_server_destroy(S);
    return st;
  }
  S->free_ranges.emplace(0, P);
  S->free_slots.reserve(c.max_inflight);
  for (int k = c.max_inflight - 1; k >= 0; --k) S->free_slots.push_back(k);
  for (int q = 0; q < fjg::kNumBuckets; ++q)
    S->limit[q] = c.oversubscribe * ctx->num_sms * std::max(1, fjg::bucket_per_sm(ctx->tune, q));
  S->limit[fjg::kLargeQueue] = std::max(1, ctx->num_sms / 2);
  *out = S;
  return FJG_OK;
}

void fjg_server_destroy(fjg_server* S) {
  if (!S) return;
  DeviceGuard dg(S->ctx->device);
  for (Lane& L : S->lanes) {
    if (L.stream) {
      cudaStreamSynchronize(L.stream);
      cudaStreamDestroy(L.stream);
    }
    if (L.ev) cudaEventDestroy(L.ev);
  }
  for (Req* r : S->pending) delete r;
  for (auto& q : S->admitted)
    for (Req* r : q) delete r;
  for (Lane& L : S->lanes)
    for (Req* r : L.batch) delete r;  // entries of completed requests are null
  for (Req* r : S->completed) delete r;
  for (auto& kv : S->returned) delete kv.second;
  if (S->copy_stream) {
    cudaStreamSynchronize(S->copy_stream);
    cudaStreamDestroy(S->copy_stream);
  }
  if (S->ev_copy) cudaEventDestroy(S->ev_copy);
  if (S->dev_mem) cudaFree(S->dev_mem);
  if (S->host_mem) cudaFreeHost(S->host_mem);
  if (S->block_mem) cudaFreeHost(S->block_mem);
  delete S;
}

fjg_status fjg_server_submit(fjg_server* S, const double* p4, int n, int algo, double r, uint64_t* ticket) {
  if (!S || !ticket) return set_error(S ? S->ctx : nullptr, FJG_EINVAL, "null argument");
  fjg_status st = check_event(S, p4, n, algo, r);
  if (st != FJG_OK) return st;
  Req* q = new (std::nothrow) Req();
  if (!q) return set_error(S->ctx, FJG_ENOMEM, "host allocation failed");
  q->n = n;
  q->algo = algo;
  q->r = r;
  q->copy.assign(p4, p4 + 4 * (size_t)n);
  q->src = q->copy.data();
  submit_req(S, q);
  *ticket = q->ticket;
  DeviceGuard dg(S->ctx->device);
  if (!progress(S)) return set_error(S->ctx, FJG_ECUDA, "server: a CUDA call failed");
  return FJG_OK;
}

fjg_status fjg_server_poll(fjg_server* S, fjg_served* out, int max, int* n_out, int64_t timeout_us) {
  if (!S || !n_out || max < 0 || (max > 0 && !out)) return set_error(S ? S->ctx : nullptr, FJG_EINVAL, "bad argument");
  *n_out = 0;
  DeviceGuard dg(S->ctx->device);
  const Clock::time_point deadline = Clock::now() + std::chrono::microseconds(timeout_us > 0 ? timeout_us : 0);
  for (;;) {
    if (!progress(S) && S->completed.empty()) return set_error(S->ctx, FJG_ECUDA, "server: a CUDA call failed");
    if (!S->completed.empty() || Clock::now() >= deadline || S->outstanding == 0) break;
  }
  int k = 0;
  while (k < max && !S->completed.empty()) {
    Req* r = S->completed.front();
    S->completed.pop_front();
    S->outstanding--;
    fjg_served& o = out[k++];
    o.ticket = r->ticket;
    o.status = r->status;
    o.n_particles = r->n;
    o.n_jets = r->n_jets;
    const int64_t s0 = r->start < 0 ? 0 : r->start;
    o.jets = S->h_jets + 4 * s0;
    o.jet_label = S->h_lab + s0;
    o.history = S->h_hist ? S->h_hist + s0 : nullptr;
    o.owner = S->h_own ? S->h_own + s0 : nullptr;
    o.latency_us = micros(r->t_done - r->t_submit);
    S->returned.emplace(r->ticket, r);
  }
  *n_out = k;
  return FJG_OK;
}

fjg_status fjg_server_release(fjg_server* S, uint64_t ticket) {
  if (!S) return set_error(nullptr, FJG_EINVAL, "server is null");
  auto it = S->returned.find(ticket);
  if (it == S->returned.end()) return set_error(S->ctx, FJG_EINVAL, "unknown or unreturned ticket");
  release_req(S, it->second);
  S->returned.erase(it);
  return FJG_OK;
}

int fjg_server_pending(const fjg_server* S) { return S ? S->outstanding : 0; }

int64_t fjg_server_launches(const fjg_server* S) { return S ? S->launches : 0; }

fjg_status fjg_server_replay(fjg_server* S, const double* p4, const int64_t* offsets, int n_events,
                             const int32_t* algo, const double* radius, const double* arrival_us,
                             double* latency_us, double* wall_us) {
  if (!S || n_events < 0 || (n_events > 0 && (!p4 || !offsets || !algo || !radius || !arrival_us || !latency_us)))
    return set_error(S ? S->ctx : nullptr, FJG_EINVAL, "bad argument");
  if (S->outstanding) return set_error(S->ctx, FJG_EAGAIN, "replay needs an idle server");
  for (int i = 0; i < n_events; ++i) {
    const int64_t n = offsets[i + 1] - offsets[i];
    if (n < 0 || n > INT32_MAX) return set_error(S->ctx, FJG_EINVAL, "bad offsets");
    fjg_status st = check_event(S, p4 + 4 * offsets[i], (int)n, algo[i], radius[i]);
    if (st != FJG_OK) return st;
    if (i > 0 && arrival_us[i] < arrival_us[i - 1]) return set_error(S->ctx, FJG_EINVAL, "arrivals must be sorted");
  }
  DeviceGuard dg(S->ctx->device);
  const Clock::time_point t0 = Clock::now();
  int next = 0, remaining = n_events, bad = 0;
  while (remaining > 0) {
    const double now_us = micros(Clock::now() - t0);
    while (next < n_events && arrival_us[next] <= now_us) {
      Req* q = new (std::nothrow) Req();
      if (!q) return set_error(S->ctx, FJG_ENOMEM, "host allocation failed");
      q->n = (int)(offsets[next + 1] - offsets[next]);
      q->algo = algo[next];
      q->r = radius[next];
      q->src = p4 + 4 * offsets[next];
      q->user = next;
      q->t_submit = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double, std::micro>(arrival_us[next]));
      submit_req(S, q);
      ++next;
    }
    if (!progress(S)) return set_error(S->ctx, FJG_ECUDA, "server: a CUDA call failed");
    while (!S->completed.empty()) {
      Req* r = S->completed.front();
      S->completed.pop_front();
      S->outstanding--;
      latency_us[r->user] = micros(r->t_done - r->t_submit);
      if (r->status != FJG_OK) ++bad;
      release_req(S, r);
      --remaining;
    }
  }
  if (wall_us) *wall_us = micros(Clock::now() - t0);
  if (bad) return set_error(S->ctx, FJG_EKERNEL, "server: some requests failed");
  return FJG_OK;
}

}  // extern "C"
