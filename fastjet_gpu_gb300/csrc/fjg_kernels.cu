// Persistent clustering kernels (one per size bucket) and the bucketing pass.
#include "fjg_kernels.cuh"

namespace fjg {

template <int T, int SPT>
__global__ void __launch_bounds__(T) k_cluster_smem(BatchArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemLayout<T, SPT>& S = *reinterpret_cast<SmemLayout<T, SPT>*>(smem_raw);
  const int count = *A.n_order;
  for (;;) {
    if (threadIdx.x == 0) {
      const int q = atomicAdd(A.queue, 1);
      S.event = (q < count) ? A.order[q] : -1;
    }
    __syncthreads();
    const int e = S.event;
    if (e < 0) break;
    cluster_event_smem<T, SPT>(S, A, e);  // ends with a barrier
  }
}

// Persistent tiled kernel for events above kSmemMaxN particles.
__global__ void __launch_bounds__(kTiledT) k_cluster_tiled(BatchArgs A) {
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
    cluster_event_tiled(S, A, A.large_ws, e);  // ends with a barrier
  }
}

// Events are handed to the bucket kernels largest first (longest-processing-
// time order), so that the biggest events do not start last and form the tail.
// Three passes: a size histogram, a descending scan that also yields each
// bucket's count, and a scatter into per-bucket lists.  Empty events are
// finished in the first pass; oversize ones raise the status word.

// Events above kSmemMaxN particles go straight to the large list (or raise
// kStatusTooBig when there is no large workspace, or it is too small).
__global__ void k_size_hist(const int64_t* offsets, int n_events, int32_t* hist, int32_t* n_jets, int* status,
                            int32_t* large_order, int32_t* large_count, int64_t large_particles) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_events; e += gridDim.x * blockDim.x) {
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
__global__ void __launch_bounds__(1024) k_size_scan(int32_t* hist, int32_t* counts) {
  __shared__ int32_t warp_sum[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // thread tid owns sizes n = kSmemMaxN - 2 tid and kSmemMaxN - 2 tid - 1 (descending)
  const int n0 = kSmemMaxN - 2 * tid, n1 = n0 - 1;
  const int h0 = hist[n0], h1 = (n1 >= 1) ? hist[n1] : 0;
  int incl = h0 + h1;
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
  const int before = incl - h0 - h1 + (warp > 0 ? warp_sum[warp - 1] : 0);  // events larger than n0
  // the start of a bucket in the descending order is the number of larger events
  const int b0 = bucket_of(n0);
  __shared__ int32_t bucket_start[kNumBuckets + 1];
  // sizes 256 << b are the largest of bucket b: their "before" is the bucket start
  for (int b = 0; b < kNumBuckets; ++b)
    if (n0 == (256 << b)) bucket_start[b] = before;
    else if (n1 == (256 << b)) bucket_start[b] = before + h0;
  if (tid == 0) bucket_start[kNumBuckets] = 0;
  __syncthreads();
  const int total = warp_sum[31];
  hist[n0] = before - bucket_start[b0];
  if (n1 >= 1) hist[n1] = before + h0 - bucket_start[bucket_of(n1)];
  if (tid < kNumBuckets) {
    // bucket b spans positions [start_b, start_{b-1}) of the descending order
    const int hi = bucket_start[tid];
    const int lo_next = (tid == 0) ? total : bucket_start[tid - 1];
    counts[tid] = lo_next - hi;
  }
}

__global__ void k_size_scatter(const int64_t* offsets, int n_events, int32_t* hist, int32_t* order, int cap_events) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_events; e += gridDim.x * blockDim.x) {
    const int64_t n64 = offsets[e + 1] - offsets[e];
    if (n64 <= 0 || n64 > kSmemMaxN) continue;
    const int pos = atomicAdd(&hist[n64], 1);
    order[bucket_of((int)n64) * cap_events + pos] = e;
  }
}

static cudaError_t launch_sort(const BatchArgs& base, const Scratch& sc, int n_events, cudaStream_t stream) {
  cudaError_t err;
  if ((err = cudaMemsetAsync(sc.hist, 0, sizeof(int32_t) * kHistBins, stream)) != cudaSuccess) return err;
  if ((err = cudaMemsetAsync(sc.queues, 0, sizeof(int) * kNumQueues, stream)) != cudaSuccess) return err;
  if ((err = cudaMemsetAsync(sc.counts + kLargeQueue, 0, sizeof(int32_t), stream)) != cudaSuccess) return err;
  const int grid = (n_events + 255) / 256 < 1 ? 1 : ((n_events + 255) / 256 > 1024 ? 1024 : (n_events + 255) / 256);
  int32_t* large_order = sc.order + kLargeQueue * sc.cap_events;
  k_size_hist<<<grid, 256, 0, stream>>>(base.offsets, n_events, sc.hist, base.n_jets, sc.status, large_order,
                                        sc.counts + kLargeQueue, sc.large_ws ? sc.large_ws_particles : 0);
  k_size_scan<<<1, 1024, 0, stream>>>(sc.hist, sc.counts);
  k_size_scatter<<<grid, 256, 0, stream>>>(base.offsets, n_events, sc.hist, sc.order, sc.cap_events);
  k_large_sort<<<1, 1024, 0, stream>>>(base.offsets, large_order, sc.counts + kLargeQueue);
  return cudaGetLastError();
}

// The large list: one CTA per event, at most two per SM (the events are
// few and long; the small buckets fill the rest of each SM).
static cudaError_t launch_large(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms,
                                cudaStream_t s) {
  if (!sc.large_ws) return cudaSuccess;
  BatchArgs A = base;
  A.order = sc.order + kLargeQueue * sc.cap_events;
  A.n_order = sc.counts + kLargeQueue;
  A.queue = sc.queues + kLargeQueue;
  A.ws = sc.ws;
  A.ws_stride = sc.ws_stride;
  A.large_ws = sc.large_ws;
  int grid = 2 * num_sms;
  if (grid > n_events) grid = n_events;
  if (grid < 1) grid = 1;
  k_cluster_tiled<<<grid, kTiledT, 0, s>>>(A);
  return cudaGetLastError();
}

template <int T, int SPT>
static cudaError_t launch_bucket(const BatchArgs& A, int grid, cudaStream_t s) {
  const size_t smem = sizeof(SmemLayout<T, SPT>);
  // the attribute is per device: set it once for each device this process uses
  static bool configured[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || !configured[dev]) {
    cudaError_t err = cudaFuncSetAttribute(k_cluster_smem<T, SPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
    if (err != cudaSuccess) return err;
    if (dev >= 0 && dev < 64) configured[dev] = true;
  }
  k_cluster_smem<T, SPT><<<grid, T, smem, s>>>(A);
  return cudaGetLastError();
}

template <int T, int SPT>
static int blocks_per_sm() {
  int nb = 0;
  const size_t smem = sizeof(SmemLayout<T, SPT>);
  cudaFuncSetAttribute(k_cluster_smem<T, SPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cluster_smem<T, SPT>, T, smem) != cudaSuccess) nb = 1;
  return nb < 1 ? 1 : nb;
}

static cudaError_t launch_bucket_dispatch(int b, const BatchArgs& A, int grid, cudaStream_t s) {
  switch (b) {
    case 0: return launch_bucket<64, 4>(A, grid, s);
    case 1: return launch_bucket<64, 8>(A, grid, s);
    case 2: return launch_bucket<128, 8>(A, grid, s);
    default: return launch_bucket<256, 8>(A, grid, s);
  }
}

static int bucket_blocks_per_sm(int b) {
  static int cache[kNumBuckets] = {0, 0, 0, 0};
  if (cache[b] == 0) {
    switch (b) {
      case 0: cache[b] = blocks_per_sm<64, 4>(); break;
      case 1: cache[b] = blocks_per_sm<64, 8>(); break;
      case 2: cache[b] = blocks_per_sm<128, 8>(); break;
      default: cache[b] = blocks_per_sm<256, 8>(); break;
    }
  }
  return cache[b];
}

cudaError_t launch_batch(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms, cudaStream_t stream,
                         cudaStream_t* side, cudaEvent_t* ev_fork, cudaEvent_t* ev_join) {
  cudaError_t err = launch_sort(base, sc, n_events, stream);
  if (err != cudaSuccess) return err;
  if ((err = cudaEventRecord(*ev_fork, stream)) != cudaSuccess) return err;
  // largest events first: their list is launched first
  {
    cudaStream_t s = side ? side[kLargeQueue] : stream;
    if (side && (err = cudaStreamWaitEvent(s, *ev_fork, 0)) != cudaSuccess) return err;
    if ((err = launch_large(base, sc, n_events, num_sms, s)) != cudaSuccess) return err;
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
    int grid = num_sms * bucket_blocks_per_sm(b);
    if (grid > n_events) grid = n_events;
    if (grid < 1) grid = 1;
    if ((err = launch_bucket_dispatch(b, A, grid, s)) != cudaSuccess) return err;
    if (side) {
      if ((err = cudaEventRecord(ev_join[b], s)) != cudaSuccess) return err;
      if ((err = cudaStreamWaitEvent(stream, ev_join[b], 0)) != cudaSuccess) return err;
    }
  }
  return cudaSuccess;
}

cudaError_t launch_batch_on_stream(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms,
                                   cudaStream_t stream) {
  cudaError_t err = launch_sort(base, sc, n_events, stream);
  if (err != cudaSuccess) return err;
  if ((err = launch_large(base, sc, n_events, num_sms, stream)) != cudaSuccess) return err;
  for (int b = kNumBuckets - 1; b >= 0; --b) {
    BatchArgs A = base;
    A.order = sc.order + b * sc.cap_events;
    A.n_order = sc.counts + b;
    A.queue = sc.queues + b;
    A.ws = sc.ws;
    A.ws_stride = sc.ws_stride;
    int grid = num_sms * bucket_blocks_per_sm(b);
    if (grid > n_events) grid = n_events;
    if (grid < 1) grid = 1;
    if ((err = launch_bucket_dispatch(b, A, grid, stream)) != cudaSuccess) return err;
  }
  return cudaSuccess;
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

cudaError_t launch_single(const BatchArgs& base, const Scratch& sc, int n, cudaStream_t stream) {
  const int b = bucket_of(n);
  if (b < 0 && (!sc.large_ws || n > sc.large_ws_particles || n > kLargeMaxN)) return cudaErrorInvalidValue;
  k_single_setup<<<1, 1, 0, stream>>>(sc.offsets1, sc.order, sc.counts, sc.queues, n);
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
    k_cluster_tiled<<<1, kTiledT, 0, stream>>>(A);
    return cudaGetLastError();
  }
  return launch_bucket_dispatch(b, A, 1, stream);
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
