// Compiled variants of the shared-memory clustering kernel (CTA size T, slots
// per thread SPT, capacity T * SPT particles) and their launchers.  The
// variants are split over two translation units so that they compile in
// parallel; the autotuner picks one per size bucket.
//
// Some shapes also have a register-capped build (__launch_bounds__ with a
// minimum of MINB resident CTAs): with 36 B of shared memory per slot more
// CTAs fit on an SM than the plain build's registers allow.  The launcher
// takes the capped build when a bucket asks for more CTAs per SM than the
// plain build fits.
#pragma once

#include "fjg_kernels.cuh"

namespace fjg {

template <int T, int SPT>
__device__ __forceinline__ void smem_event_loop(const BatchArgs& A) {
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
    if (refused_event(A, e)) continue;  // ends with a barrier
    cluster_event_smem<T, SPT>(S, A, e);  // ends with a barrier
    if (threadIdx.x == 0) signal_done(A, e);
  }
}

template <int T, int SPT>
__global__ void __launch_bounds__(T) k_cluster_smem(BatchArgs A) {
  smem_event_loop<T, SPT>(A);
}

template <int T, int SPT, int MINB>
__global__ void __launch_bounds__(T, MINB) k_cluster_smem_capped(BatchArgs A) {
  smem_event_loop<T, SPT>(A);
}

// Dynamic shared memory attribute, set once per device and kernel.
template <class K>
cudaError_t configure_smem(K kernel, size_t bytes, bool* configured) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev >= 0 && dev < 64 && configured[dev]) return cudaSuccess;
  err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err == cudaSuccess && dev >= 0 && dev < 64) configured[dev] = true;
  return err;
}

template <class K>
int occupancy_of(K kernel, int threads, size_t bytes, bool* configured) {
  if (configure_smem(kernel, bytes, configured) != cudaSuccess) return 1;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, bytes) != cudaSuccess) nb = 1;
  return nb < 1 ? 1 : nb;
}

// Per-kernel "attribute set" flags, shared by the occupancy query and the
// launcher, so that a launch inside a stream capture finds them set.
template <int T, int SPT>
bool* smem_configured() {
  static bool f[64] = {};
  return f;
}

template <int T, int SPT, int MINB>
bool* smem_configured_capped() {
  static bool f[64] = {};
  return f;
}

template <int T, int SPT>
cudaError_t launch_smem(const BatchArgs& A, int grid, cudaStream_t s) {
  cudaError_t err = configure_smem(k_cluster_smem<T, SPT>, sizeof(SmemLayout<T, SPT>), smem_configured<T, SPT>());
  if (err != cudaSuccess) return err;
  return launch_with_priority(k_cluster_smem<T, SPT>, grid, T, sizeof(SmemLayout<T, SPT>), s,
                              bucket_priority_level(bucket_of(T * SPT), A.serve_order), A);
}

template <int T, int SPT, int MINB>
cudaError_t launch_smem_capped(const BatchArgs& A, int grid, cudaStream_t s) {
  cudaError_t err = configure_smem(k_cluster_smem_capped<T, SPT, MINB>, sizeof(SmemLayout<T, SPT>),
                                   smem_configured_capped<T, SPT, MINB>());
  if (err != cudaSuccess) return err;
  return launch_with_priority(k_cluster_smem_capped<T, SPT, MINB>, grid, T, sizeof(SmemLayout<T, SPT>), s,
                              bucket_priority_level(bucket_of(T * SPT), A.serve_order), A);
}

template <int T, int SPT>
int occupancy_smem() {
  return occupancy_of(k_cluster_smem<T, SPT>, T, sizeof(SmemLayout<T, SPT>), smem_configured<T, SPT>());
}

template <int T, int SPT, int MINB>
int occupancy_smem_capped() {
  return occupancy_of(k_cluster_smem_capped<T, SPT, MINB>, T, sizeof(SmemLayout<T, SPT>),
                      smem_configured_capped<T, SPT, MINB>());
}

// Variants compiled in each translation unit (v in [0, kNumVariants)):
// launch one (the capped build when `capped` and the shape has one), or
// report its resident CTAs per SM; -1 / cudaErrorInvalidValue for a variant
// the unit does not hold.
cudaError_t launch_variant_small(int v, const BatchArgs& A, int grid, bool capped, cudaStream_t s);
int occupancy_variant_small(int v, bool capped);
cudaError_t launch_variant_large(int v, const BatchArgs& A, int grid, bool capped, cudaStream_t s);
int occupancy_variant_large(int v, bool capped);

}  // namespace fjg
