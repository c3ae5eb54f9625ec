// Kernel entry points and launch helpers shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include "fjg_cluster.cuh"
#include "fjg_cluster_tiled.cuh"

namespace fjg {

// Size buckets of the shared-memory path: bucket b holds events of up to
// 256 << b particles (36 bytes of shared memory per slot; by default CTAs of
// 64, 64, 128, 256 and 512 threads with 4, 8, 8, 8 and 8 slots per thread;
// with the register-capped builds 12, 10, 5, 3 and 1 of them share an SM).
constexpr int kNumBuckets = 5;
constexpr int kSmemMaxN = 4096;
// Events above kSmemMaxN particles form one more work list, run by the tiled
// kernel (one CTA of 256 threads per event, state in the large workspace).
constexpr int kLargeQueue = kNumBuckets;
constexpr int kNumQueues = kNumBuckets + 1;
constexpr int kLargeMaxN = 1 << 24;

__host__ __device__ inline int bucket_of(int n) {
  return n <= 256 ? 0 : n <= 512 ? 1 : n <= 1024 ? 2 : n <= 2048 ? 3 : n <= 4096 ? 4 : -1;
}

// R accepted by the entry points: finite and >= 0.  R = 0 is allowed, as the
// reference driver allows it (main.cc:159): 1/R^2 is then infinite, every pair
// distance is infinite (NaN for coincident pseudojets, which never undercuts a
// beam distance either), so every particle is promoted to a jet in order of
// its weight -- what the reference's cluster() computes (tri_matrix.cu:305).
inline bool valid_radius(double r) { return r >= 0.0 && r <= 1.7976931348623157e308; }

// Compiled variants of the shared-memory kernel: CTA size and slots per
// thread (capacity = their product).  A bucket of capacity 256 << b can run
// any variant of exactly that capacity.
constexpr int kNumVariants = 11;
struct VariantShape {
  int threads, spt;
};
__host__ __device__ inline VariantShape variant_shape(int v) {
  switch (v) {
    case 0: return {64, 4};
    case 1: return {128, 2};
    case 2: return {64, 8};
    case 3: return {128, 4};
    case 4: return {256, 2};
    case 5: return {128, 8};
    case 6: return {256, 4};
    case 7: return {256, 8};
    case 8: return {512, 4};
    case 9: return {512, 8};
    case 10: return {256, 16};
    default: return {0, 0};
  }
}

// Launch configuration the autotuner chooses: per bucket a variant and the
// CTAs per SM of its persistent grid (0: as many as fit), the CTAs per SM of
// the tiled kernel, and its tile side in units of R (>= 1).
struct BucketConfig {
  int variant;
  int ctas_per_sm;
};
struct Tuning {
  BucketConfig bucket[kNumBuckets];
  int large_ctas_per_sm;
  double tile_factor;
};
inline Tuning default_tuning() { return Tuning{{{0, 0}, {2, 0}, {5, 0}, {7, 0}, {9, 0}}, 2, 1.0}; }
bool tuning_valid(const Tuning& t);

// Scheduling priority of a clustering launch: level 0 (the tiled kernel) is
// the most urgent, then the size buckets from the largest down
// (level kNumBuckets - b), so that when the bucket kernels of one batch run
// side by side the SMs take the longest events first and the small buckets
// fill the tail.  Levels beyond the device's range share its lowest priority.
// A request server wants the opposite (`serve_order`): its small events are
// the latency-bound ones, so they go first and the tiled kernel last.
int launch_priority(int level);
inline int bucket_priority_level(int b, int serve_order) { return serve_order ? b : kNumBuckets - b; }
inline int tiled_priority_level(int serve_order) { return serve_order ? kNumBuckets : 0; }

// Launch of a clustering kernel with its priority as a launch attribute
// (recorded in a captured graph too).
template <class K>
cudaError_t launch_with_priority(K kernel, int grid, int threads, size_t smem, cudaStream_t s, int level,
                                 const BatchArgs& A) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid < 1 ? 1 : grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = launch_priority(level);
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, A);
}

// The tiled kernel over the work list of A (a persistent grid of `grid` CTAs).
cudaError_t launch_tiled(const BatchArgs& A, int grid, cudaStream_t s);
// Sets the tiled kernel's launch attributes once per device (outside a capture).
cudaError_t configure_tiled();

// Launch variant v (a persistent grid of `grid` CTAs); resident CTAs per SM of
// variant v on the current device.
cudaError_t launch_variant(int v, const BatchArgs& A, int grid, int per_sm, cudaStream_t s);
int variant_occupancy(int v);        // most CTAs per SM of any build of variant v
int variant_occupancy_plain(int v);  // of its plain build (more takes the register-capped one)
int bucket_per_sm(const Tuning& tune, int b);  // CTAs per SM that bucket b runs with

// Device-side batch descriptor scratch owned by a context.
struct Scratch {
  int32_t* order;   // [kNumQueues][cap_events]
  int32_t* counts;  // [kNumQueues]
  int* queues;      // [kNumQueues]
  int* status;      // [1]
  int64_t* offsets1;  // [2] single-event offsets {0, n}
  int cap_events;
  double* ws;         // [kWsFields][ws_stride] exact per-particle state
  int64_t ws_stride;  // particles the workspace holds
  int32_t* hist;      // [kHistBins] events per size, then per-size positions (sorting by size)
  unsigned char* large_ws;    // kLargeWsBytesPerParticle per particle, 16 B aligned (null: large events are refused)
  int64_t large_ws_particles;  // particles the large workspace covers
};

constexpr int kHistBins = kSmemMaxN + 1;

// Launch the bucketing kernels plus one persistent kernel per work list on
// `stream` (the lists run concurrently on the kNumQueues side streams when
// given).
cudaError_t launch_batch(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms, const Tuning& tune,
                         cudaStream_t stream, cudaStream_t* side, cudaEvent_t* ev_fork, cudaEvent_t* ev_join);

// The bucketing kernels and the per-list kernels, all on `stream` one after
// another (no side streams, no events).
cudaError_t launch_batch_on_stream(const BatchArgs& base, const Scratch& sc, int n_events, int num_sms,
                                   const Tuning& tune, cudaStream_t stream);

// One event, one CTA (the plain per-event-launch path; the tiled kernel above
// kSmemMaxN particles).
cudaError_t launch_single(const BatchArgs& base, const Scratch& sc, int n, const Tuning& tune, cudaStream_t stream);

// Finiteness check of a request server's micro-batch ((start, end) pairs of
// [n][4] momenta): bad events get kStatusBadArg in ev_status.
cudaError_t launch_check_pairs(const double* p4, const int64_t* pairs, int n_events, int32_t* ev_status,
                               cudaStream_t s);

// Scatter jets into the reference's PseudoJet records (in place).
cudaError_t launch_pseudojet_epilogue(void* records, int size, const double* jets, const int32_t* jet_label,
                                      const int32_t* n_jets, cudaStream_t stream);

// Rapidity, azimuth and weight of n four-momenta (the clustering kernels' own
// kinematics routine, one thread per particle).
cudaError_t launch_kinematics(const double* p4, int n, int algo, double* rap, double* phi, double* w,
                              cudaStream_t stream);

// Record a message as the calling thread's last error (fjg_last_error(NULL)).
void set_thread_error(const char* msg);

}  // namespace fjg
