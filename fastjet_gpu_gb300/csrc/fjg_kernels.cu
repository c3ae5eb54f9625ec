// Persistent clustering kernels (one per size bucket) and the bucketing pass.
#include "fjg_kernels.cuh"
#include "fjg_variants.cuh"

namespace fjg {

// Persistent tiled kernel for events above kSmemMaxN particles.
__global__ void __launch_bounds__(kTiledT, 1) k_cluster_tiled(BatchArgs A) {
  __shared__ TiledShared S;
  const int count = *A.n_order;
  for (;;) {
    if (threadIdx.x == 0) {
      const int q = atomicAdd(A.queue, 1);
      S.event = (q < count) ? A.order[q] : -1;
    }
    __syncthreads();
    const int e = S.event;
    if (e < 0) break;
    if (refused_event(A, e)) continue;  // ends with a barrier
    cluster_event_tiled(S, A, A.large_ws, e);  // ends with a barrier
    if (threadIdx.x == 0) signal_done(A, e);
  }
}

int launch_priority(int level) {
  static int range[64][3] = {};  // resolved, least, greatest
  int dev = 0;
  cudaGetDevice(&dev);
  int least = 0, greatest = 0;
  if (dev >= 0 && dev < 64 && range[dev][0]) {
    least = range[dev][1];
    greatest = range[dev][2];
  } else if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess && dev >= 0 && dev < 64) {
    range[dev][0] = 1;
    range[dev][1] = least;
    range[dev][2] = greatest;
  }
  // numerically lower is more urgent: greatest <= least
  const int p = greatest + level;
  return p > least ? least : p;
}

// The tiled kernel keeps its per-slot state in global memory and leans on L1
// (its 46 KB of shared memory hold the tile ranges and summaries): ask for the
// largest L1 split, so that it does not run with the small L1 that the
// shared-memory bucket kernels leave on an SM.
cudaError_t configure_tiled() {
  static bool done[64] = {};
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
  err = cudaFuncSetAttribute(k_cluster_tiled, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxL1);
  if (err == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
  return err;
}

cudaError_t launch_tiled(const BatchArgs& A, int grid, cudaStream_t s) {
  cudaError_t err = configure_tiled();
  if (err != cudaSuccess) return err;
  return launch_with_priority(k_cluster_tiled, grid, kTiledT, 0, s, tiled_priority_level(A.serve_order), A);
}

// Events are handed to the bucket kernels largest first (longest-processing-
// time order), so that the biggest events do not start last and form the tail.
// Three passes: a size histogram, a descending scan that also yields each
// bucket's count, and a scatter into per-bucket lists.  Empty events are
// finished in the first pass; oversize ones raise the status word.

// Events above kSmemMaxN particles go straight to the large list (or raise
// kStatusTooBig when there is no large workspace, or it is too small).
// Input check, in two launches.  `limit` is the smaller of the caller's
// particle count (the size of p4) and the workspace the kernels index by the
// same offsets.  k_check_args, one thread per event: n_jets[e] = -1 when the
// event's particle range does not lie inside [0, limit), or its algorithm code
// (per-event array) is not kt, C/A or anti-kt, or its R (per-event array) is
// not finite and >= 0; else 0.  k_check_moms, a flat pass over every momentum
// of [offsets[0], min(offsets[n_events], limit)) (16-byte loads where the
// layout allows): an event with a NaN or infinite component gets n_jets[e] =
// -1 (its event is found by a binary search of the offsets; such events are
// rare).  No momentum past `limit` is read, whatever the offsets say.  Refused events raise
// kStatusBadArg in k_size_hist and get no jets.  Events of no or too many
// particles are left to the bucketing.
__global__ void k_check_args(const int64_t* offsets, int n_events, int32_t* n_jets, int64_t limit,
                             const int32_t* algo, const double* radius) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_events; e += gridDim.x * blockDim.x) {
    const int64_t o0 = offsets[e], o1 = offsets[e + 1];
    bool bad = o1 > o0 && (o0 < 0 || o1 > limit);
    if (algo) bad |= algo[e] < -1 || algo[e] > 1;
    if (radius) bad |= !(radius[e] >= 0.0 && isfinite(radius[e]));
    n_jets[e] = bad ? -1 : 0;
  }
}

__device__ __forceinline__ int event_of(const int64_t* offsets, int n_events, int64_t s) {
  int lo = 0, hi = n_events - 1;  // the last event with offsets[e] <= s
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= s) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// vec: p4 is [n][4] doubles on a 16-byte boundary, read as pairs of doubles.
__global__ void k_check_moms(const double* p4, int p4_stride, const int64_t* offsets, int n_events,
                             int32_t* n_jets, int64_t limit, int vec) {
  // the particles of the batch, [offsets[0], offsets[n_events]), inside p4 and the workspace
  int64_t end = offsets[n_events];
  end = end < limit ? end : limit;
  const int64_t begin = offsets[0] > 0 ? offsets[0] : 0;
  if (end <= begin) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (vec) {
    // four independent 16-byte loads in flight per thread and iteration
    const double2* q = reinterpret_cast<const double2*>(p4);
    const int64_t lim = 2 * end;
    for (int64_t i = 2 * begin + first; i < lim; i += 4 * stride) {
      double2 v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = (i + k * stride < lim) ? __ldg(q + i + k * stride) : make_double2(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (!(isfinite(v[k].x) && isfinite(v[k].y))) n_jets[event_of(offsets, n_events, (i + k * stride) >> 1)] = -1;
    }
  } else {
    for (int64_t s = begin + first; s < end; s += stride) {
      const double* p = p4 + s * p4_stride;
      if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]) && isfinite(p[3])))
        n_jets[event_of(offsets, n_events, s)] = -1;
    }
  }
}

// Input check of a request server's micro-batch ((start, end) pairs), one
// warp per event: an event with a non-finite momentum component gets
// kStatusBadArg in its own status word, so the clustering kernel skips it and
// only its request fails.
__global__ void k_check_pairs(const double* p4, const int64_t* pairs, int n_events, int32_t* ev_status) {
  const int lane = threadIdx.x & 31;
  const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int e = w0; e < n_events; e += nw) {
    const int64_t o0 = pairs[2 * (int64_t)e], o1 = pairs[2 * (int64_t)e + 1];
    bool bad = false;
    for (int64_t s = o0 + lane; s < o1; s += 32) {
      const double* p = p4 + 4 * s;
      bad |= !(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]) && isfinite(p[3]));
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) ev_status[e] |= kStatusBadArg;
  }
}

cudaError_t launch_check_pairs(const double* p4, const int64_t* pairs, int n_events, int32_t* ev_status,
                               cudaStream_t s) {
  const int grid = (n_events + 7) / 8 > 1024 ? 1024 : (n_events + 7) / 8;  // 8 events (warps) per block
  k_check_pairs<<<grid < 1 ? 1 : grid, 256, 0, s>>>(p4, pairs, n_events, ev_status);
  return cudaGetLastError();
}

__global__ void k_size_hist(const int64_t* offsets, int n_events, int32_t* hist, int32_t* n_jets, int* status,
                            int32_t* large_order, int32_t* large_count, int64_t large_particles) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_events; e += gridDim.x * blockDim.x) {
    if (n_jets[e] < 0) {  // refused by the input check (k_check_args, k_check_moms); k_size_scatter resets it
      atomicOr(status, kStatusBadArg);
      continue;
    }
    const int64_t n64 = offsets[e + 1] - offsets[e];
    if (n64 > kSmemMaxN) {
      if (n64 <= kLargeMaxN && offsets[e + 1] <= large_particles) {
        large_order[atomicAdd(large_count, 1)] = e;
      } else {
        n_jets[e] = 0;
        atomicOr(status, kStatusTooBig);
      }
      continue;
    }
    if (n64 <= 0) {
      n_jets[e] = 0;
      if (n64 < 0) atomicOr(status, kStatusBadArg);
      continue;
    }
    atomicAdd(&hist[n64], 1);
  }
}

// Largest first within the large list (rank sort in one block; lists longer
// than kLargeSortMax keep their arrival order, which is only slower).
constexpr int kLargeSortMax = 4096;

__global__ void __launch_bounds__(1024) k_large_sort(const int64_t* offsets, int32_t* order, const int32_t* count) {
  __shared__ int32_t ev[kLargeSortMax];
  __shared__ int32_t sz[kLargeSortMax];
  const int L = *count;
  if (L < 2 || L > kLargeSortMax) return;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const int e = order[i];
    ev[i] = e;
    sz[i] = (int)(offsets[e + 1] - offsets[e]);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    int rank = 0;
    for (int k = 0; k < L; ++k) rank += (sz[k] > sz[i]) || (sz[k] == sz[i] && ev[k] < ev[i]);
    order[rank] = ev[i];
  }
}

// One block of 1024 threads: hist[n] becomes the position of the first event
// of size n inside its bucket's list (sizes in descending order), counts[b]
// the number of events of bucket b.
constexpr int kScanPerThread = kSmemMaxN / 1024;

__global__ void __launch_bounds__(1024) k_size_scan(int32_t* hist, int32_t* counts) {
  __shared__ int32_t warp_sum[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // thread tid owns sizes n = kSmemMaxN - kScanPerThread * tid - k (descending)
  const int n_first = kSmemMaxN - kScanPerThread * tid;
  int h[kScanPerThread];
  int mine = 0;
  for (int k = 0; k < kScanPerThread; ++k) {
    const int n = n_first - k;
    h[k] = (n >= 1) ? hist[n] : 0;
    mine += h[k];
  }
  int incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = warp_sum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    warp_sum[lane] = v;
  }
  __syncthreads();
  // events larger than size n_first - k, for each k
  int before[kScanPerThread];
  before[0] = incl - mine + (warp > 0 ? warp_sum[warp - 1] : 0);
  for (int k = 1; k < kScanPerThread; ++k) before[k] = before[k - 1] + h[k - 1];
  // the start of a bucket in the descending order is the number of larger
  // events; sizes 256 << b are the largest of bucket b
  __shared__ int32_t bucket_start[kNumBuckets + 1];
  for (int k = 0; k < kScanPerThread; ++k)
    for (int b = 0; b < kNumBuckets; ++b)
      if (n_first - k == (256 << b)) bucket_start[b] = before[k];
  if (tid == 0) bucket_start[kNumBuckets] = 0;
  __syncthreads();
  const int total = warp_sum[31];
  for (int k = 0; k < kScanPerThread; ++k) {
    const int n = n_first - k;
    if (n >= 1) hist[n] = before[k] - bucket_start[bucket_of(n)];
  }
  if (tid < kNumBuckets) {
    // bucket b spans positions [start_b, start_{b-1}) of the descending order
    const int hi = bucket_start[tid];
    const int lo_next = (tid == 0) ? total : bucket_start[tid - 1];
    counts[tid] = lo_next - hi;
  }
}

__global__ void k_size_scatter(const int64_t* offsets, int n_events, int32_t* hist, int32_t* order, int cap_events,
                               int32_t* n_jets) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_events; e += gridDim.x * blockDim.x) {
    if (n_jets[e] < 0) {  // refused: no jets
      n_jets[e] = 0;
      continue;
    }
    const int64_t n64 = offsets[e + 1] - offsets[e];
    if (n64 <= 0 || n64 > kSmemMaxN) continue;
    const int pos = atomicAdd(&hist[n64], 1);
    order[bucket_of((int)n64) * cap_events + pos] = e;
  }
}

// Blocks of the momentum check: a few per SM, enough 16-byte loads in flight
// to approach the HBM bandwidth, grid-stride over the rest.
static int check_grid() {
  static int cache[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && cache[dev]) return cache[dev];
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 132;
  const int g = 8 * sms;
  if (dev >= 0 && dev < 64) cache[dev] = g;
  return g;
}

static cudaError_t launch_sort(const BatchArgs& base, const Scratch& sc, int n_events, cudaStream_t stream) {
  cudaError_t err;
  if ((err = cudaMemsetAsync(sc.hist, 0, sizeof(int32_t) * kHistBins, stream)) != cudaSuccess) return err;
  if ((err = cudaMemsetAsync(sc.queues, 0, sizeof(int) * kNumQueues, stream)) != cudaSuccess) return err;
  if ((err = cudaMemsetAsync(sc.counts + kLargeQueue, 0, sizeof(int32_t), stream)) != cudaSuccess) return err;
  const int grid = (n_events + 255) / 256 < 1 ? 1 : ((n_events + 255) / 256 > 1024 ? 1024 : (n_events + 255) / 256);
  const int64_t limit = base.particles < sc.ws_stride ? base.particles : sc.ws_stride;
  k_check_args<<<grid, 256, 0, stream>>>(base.offsets, n_events, base.n_jets, limit, base.algo, base.radius);
  const int vec = base.p4_stride == 4 && (reinterpret_cast<uintptr_t>(base.p4) & 15) == 0;
  k_check_moms<<<check_grid(), 256, 0, stream>>>(base.p4, base.p4_stride, base.offsets, n_events, base.n_jets,
                                                 limit, vec);
  int32_t* large_order = sc.order + kLargeQueue * sc.cap_events;
  k_size_hist<<<grid, 256, 0, stream>>>(base.offsets, n_events, sc.hist, base.n_jets, sc.status, large_order,
                                        sc.counts + kLargeQueue, sc.large_ws ? sc.large_ws_particles : 0);
  k_size_scan<<<1, 1024, 0, stream>>>(sc.hist, sc.counts);
  k_size_scatter<<<grid, 256, 0, stream>>>(base.offsets, n_events, sc.hist, sc.order, sc.cap_events, base.n_jets);
  k_large_sort<<<1, 1024, 0, stream>>>(base.offsets, large_order, sc.counts + kLargeQueue);
  return cudaGetLastError();
}

// The large list: one CTA per event, a few per SM at most (the events are
// few and long; the small buckets fill the rest of each SM).
static cudaError_t launch_large(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms,
                                const Tuning& tune, cudaStream_t s) {
  if (!sc.large_ws) return cudaSuccess;
  BatchArgs A = base;
  A.order = sc.order + kLargeQueue * sc.cap_events;
  A.n_order = sc.counts + kLargeQueue;
  A.queue = sc.queues + kLargeQueue;
  A.ws = sc.ws;
  A.ws_stride = sc.ws_stride;
  A.large_ws = sc.large_ws;
  A.tile_factor = tune.tile_factor;
  int grid = tune.large_ctas_per_sm * num_sms;
  if (grid > n_events) grid = n_events;
  if (grid < 1) grid = 1;
  cudaError_t err = configure_tiled();
  if (err != cudaSuccess) return err;
  k_cluster_tiled<<<grid, kTiledT, 0, s>>>(A);
  return cudaGetLastError();
}

bool tuning_valid(const Tuning& t) {
  for (int b = 0; b < kNumBuckets; ++b) {
    const int v = t.bucket[b].variant;
    if (v < 0 || v >= kNumVariants) return false;
    const VariantShape sh = variant_shape(v);
    if (sh.threads * sh.spt != (256 << b)) return false;
    if (t.bucket[b].ctas_per_sm < 0 || t.bucket[b].ctas_per_sm > 64) return false;
  }
  return t.large_ctas_per_sm >= 1 && t.large_ctas_per_sm <= 8 && t.tile_factor >= 1.0 && t.tile_factor <= 8.0;
}

static int occupancy_cached(int v, bool capped) {
  static int cache[64][kNumVariants][2] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  int* slot = (dev >= 0 && dev < 64 && v >= 0 && v < kNumVariants) ? &cache[dev][v][capped ? 1 : 0] : nullptr;
  if (slot && *slot > 0) return *slot;
  int nb = occupancy_variant_small(v, capped);
  if (nb < 0) nb = occupancy_variant_large(v, capped);
  if (nb < 1) nb = 1;
  if (slot) *slot = nb;
  return nb;
}

int variant_occupancy_plain(int v) { return occupancy_cached(v, false); }

int variant_occupancy(int v) {
  const int plain = occupancy_cached(v, false), capped = occupancy_cached(v, true);
  return plain > capped ? plain : capped;
}

cudaError_t launch_variant(int v, const BatchArgs& A, int grid, int per_sm, cudaStream_t s) {
  const bool capped = per_sm > variant_occupancy_plain(v);
  cudaError_t err = launch_variant_small(v, A, grid, capped, s);
  if (err == cudaErrorInvalidValue) err = launch_variant_large(v, A, grid, capped, s);
  return err;
}

// Persistent grid of bucket b: the configured CTAs per SM (0: as many as the
// plain build fits), at most what any build fits, at most one CTA per event.
int bucket_per_sm(const Tuning& tune, int b) {
  const int v = tune.bucket[b].variant;
  const int per_sm = tune.bucket[b].ctas_per_sm;
  if (per_sm <= 0) return variant_occupancy_plain(v);
  const int fit = variant_occupancy(v);
  return per_sm > fit ? fit : per_sm;
}

static int bucket_grid(const Tuning& tune, int b, int num_sms, int n_events) {
  int grid = num_sms * bucket_per_sm(tune, b);
  if (grid > n_events) grid = n_events;
  return grid < 1 ? 1 : grid;
}

cudaError_t launch_batch(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms, const Tuning& tune,
                         cudaStream_t stream, cudaStream_t* side, cudaEvent_t* ev_fork, cudaEvent_t* ev_join) {
  cudaError_t err = launch_sort(base, sc, n_events, stream);
  if (err != cudaSuccess) return err;
  if ((err = cudaEventRecord(*ev_fork, stream)) != cudaSuccess) return err;
  // largest events first: their list is launched first
  {
    cudaStream_t s = side ? side[kLargeQueue] : stream;
    if (side && (err = cudaStreamWaitEvent(s, *ev_fork, 0)) != cudaSuccess) return err;
    if ((err = launch_large(base, sc, n_events, num_sms, tune, s)) != cudaSuccess) return err;
    if (side) {
      if ((err = cudaEventRecord(ev_join[kLargeQueue], s)) != cudaSuccess) return err;
      if ((err = cudaStreamWaitEvent(stream, ev_join[kLargeQueue], 0)) != cudaSuccess) return err;
    }
  }
  for (int b = kNumBuckets - 1; b >= 0; --b) {
    cudaStream_t s = side ? side[b] : stream;
    if (side && (err = cudaStreamWaitEvent(s, *ev_fork, 0)) != cudaSuccess) return err;
    BatchArgs A = base;
    A.order = sc.order + b * sc.cap_events;
    A.n_order = sc.counts + b;
    A.queue = sc.queues + b;
    A.ws = sc.ws;
    A.ws_stride = sc.ws_stride;
    if ((err = launch_variant(tune.bucket[b].variant, A, bucket_grid(tune, b, num_sms, n_events),
                              bucket_per_sm(tune, b), s)) != cudaSuccess)
      return err;
    if (side) {
      if ((err = cudaEventRecord(ev_join[b], s)) != cudaSuccess) return err;
      if ((err = cudaStreamWaitEvent(stream, ev_join[b], 0)) != cudaSuccess) return err;
    }
  }
  return cudaSuccess;
}

cudaError_t launch_batch_on_stream(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms,
                                   const Tuning& tune, cudaStream_t stream) {
  cudaError_t err = launch_sort(base, sc, n_events, stream);
  if (err != cudaSuccess) return err;
  if ((err = launch_large(base, sc, n_events, num_sms, tune, stream)) != cudaSuccess) return err;
  for (int b = kNumBuckets - 1; b >= 0; --b) {
    BatchArgs A = base;
    A.order = sc.order + b * sc.cap_events;
    A.n_order = sc.counts + b;
    A.queue = sc.queues + b;
    A.ws = sc.ws;
    A.ws_stride = sc.ws_stride;
    if ((err = launch_variant(tune.bucket[b].variant, A, bucket_grid(tune, b, num_sms, n_events),
                              bucket_per_sm(tune, b), stream)) != cudaSuccess)
      return err;
  }
  return cudaSuccess;
}

// The single-event path's input check: an event with a non-finite momentum
// empties every work list (nothing runs) and raises kStatusBadArg.
__global__ void k_check_single(const double* p4, int p4_stride, int n, int32_t* counts, int32_t* n_jets,
                               int* status) {
  __shared__ int any_bad;
  if (threadIdx.x == 0) any_bad = 0;
  __syncthreads();
  bool bad = false;
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    const double* p = p4 + (int64_t)s * p4_stride;
    bad |= !(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]) && isfinite(p[3]));
  }
  if (bad) any_bad = 1;
  __syncthreads();
  if (threadIdx.x == 0 && any_bad) {
    for (int b = 0; b < kNumQueues; ++b) counts[b] = 0;
    n_jets[0] = 0;
    atomicOr(status, kStatusBadArg);
  }
}

__global__ void k_single_setup(int64_t* offsets1, int32_t* order, int32_t* counts, int* queues, int n) {
  offsets1[0] = 0;
  offsets1[1] = n;
  order[0] = 0;
  for (int b = 0; b < kNumQueues; ++b) {
    counts[b] = 1;
    queues[b] = 0;
  }
}

cudaError_t launch_single(const BatchArgs& base, const Scratch& sc, int n, const Tuning& tune, cudaStream_t stream) {
  const int b = bucket_of(n);
  if (b < 0 && (!sc.large_ws || n > sc.large_ws_particles || n > kLargeMaxN)) return cudaErrorInvalidValue;
  k_single_setup<<<1, 1, 0, stream>>>(sc.offsets1, sc.order, sc.counts, sc.queues, n);
  k_check_single<<<1, 256, 0, stream>>>(base.p4, base.p4_stride, n, sc.counts, base.n_jets, sc.status);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  BatchArgs A = base;
  A.offsets = sc.offsets1;
  A.order = sc.order;
  A.n_order = sc.counts;
  A.queue = sc.queues;
  A.ws = sc.ws;
  A.ws_stride = sc.ws_stride;
  if (b < 0) {
    A.large_ws = sc.large_ws;
    A.tile_factor = tune.tile_factor;
    if ((err = configure_tiled()) != cudaSuccess) return err;
    k_cluster_tiled<<<1, kTiledT, 0, stream>>>(A);
    return cudaGetLastError();
  }
  return launch_variant(tune.bucket[b].variant, A, 1, 1, stream);
}

__global__ void k_kinematics(const double* p4, int n, int algo, double* rap, double* phi, double* w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const Kin k = kinematics(p4[4 * i + 0], p4[4 * i + 1], p4[4 * i + 2], p4[4 * i + 3], algo);
    rap[i] = k.rap;
    phi[i] = k.phi;
    w[i] = k.w;
  }
}

cudaError_t launch_kinematics(const double* p4, int n, int algo, double* rap, double* phi, double* w,
                              cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int grid = (n + 255) / 256 > 4096 ? 4096 : (n + 255) / 256;
  k_kinematics<<<grid, 256, 0, stream>>>(p4, n, algo, rap, phi, w);
  return cudaGetLastError();
}

// PseudoJet record (PseudoJet.h:4-11): int index; bool isJet; double px, py, pz, E.
struct PJRecord {
  int index;
  bool isJet;
  double px, py, pz, E;
};
static_assert(sizeof(PJRecord) == 40, "PseudoJet layout");

__global__ void k_pj_reset(PJRecord* rec, int size) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < size; s += gridDim.x * blockDim.x) {
    rec[s].index = s;
    rec[s].isJet = false;
  }
}

__global__ void k_pj_scatter(PJRecord* rec, const double* jets, const int32_t* jet_label, const int32_t* n_jets) {
  const int nj = *n_jets;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nj; k += gridDim.x * blockDim.x) {
    const int s = jet_label[k];
    rec[s].px = jets[4 * k + 0];
    rec[s].py = jets[4 * k + 1];
    rec[s].pz = jets[4 * k + 2];
    rec[s].E = jets[4 * k + 3];
    rec[s].isJet = true;
  }
}

cudaError_t launch_pseudojet_epilogue(void* records, int size, const double* jets, const int32_t* jet_label,
                                      const int32_t* n_jets, cudaStream_t stream) {
  if (size <= 0) return cudaSuccess;
  const int grid = (size + 255) / 256 > 256 ? 256 : (size + 255) / 256;
  k_pj_reset<<<grid, 256, 0, stream>>>(reinterpret_cast<PJRecord*>(records), size);
  k_pj_scatter<<<grid, 256, 0, stream>>>(reinterpret_cast<PJRecord*>(records), jets, jet_label, n_jets);
  return cudaGetLastError();
}

}  // namespace fjg
