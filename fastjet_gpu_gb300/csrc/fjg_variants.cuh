// Compiled variants of the shared-memory clustering kernel (CTA size T, slots
// per thread SPT, capacity T * SPT particles) and their launchers.  The
// variants are split over two translation units so that they compile in
// parallel; the autotuner picks one per size bucket.
#pragma once

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
    if (threadIdx.x == 0) signal_done(A, e);
  }
}

// Dynamic shared memory attribute, set once per device and variant.
template <int T, int SPT>
cudaError_t configure_smem() {
  static bool configured[64] = {};
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev >= 0 && dev < 64 && configured[dev]) return cudaSuccess;
  err = cudaFuncSetAttribute(k_cluster_smem<T, SPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(SmemLayout<T, SPT>));
  if (err == cudaSuccess && dev >= 0 && dev < 64) configured[dev] = true;
  return err;
}

template <int T, int SPT>
cudaError_t launch_smem(const BatchArgs& A, int grid, cudaStream_t s) {
  cudaError_t err = configure_smem<T, SPT>();
  if (err != cudaSuccess) return err;
  k_cluster_smem<T, SPT><<<grid, T, sizeof(SmemLayout<T, SPT>), s>>>(A);
  return cudaGetLastError();
}

template <int T, int SPT>
int occupancy_smem() {
  if (configure_smem<T, SPT>() != cudaSuccess) return 1;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cluster_smem<T, SPT>, T, sizeof(SmemLayout<T, SPT>)) !=
      cudaSuccess)
    nb = 1;
  return nb < 1 ? 1 : nb;
}

// Variants compiled in each translation unit (v in [0, kNumVariants)):
// launch one, or report its resident CTAs per SM; -1 / cudaErrorInvalidValue
// for a variant the unit does not hold.
cudaError_t launch_variant_small(int v, const BatchArgs& A, int grid, cudaStream_t s);
int occupancy_variant_small(int v);
cudaError_t launch_variant_large(int v, const BatchArgs& A, int grid, cudaStream_t s);
int occupancy_variant_large(int v);

}  // namespace fjg
