// Shared-memory kernel variants of capacity 256 and 512 particles.
#include "fjg_variants.cuh"

namespace fjg {

cudaError_t launch_variant_small(int v, const BatchArgs& A, int grid, bool capped, cudaStream_t s) {
  switch (v) {
    case 0: return capped ? launch_smem_capped<64, 4, 12>(A, grid, s) : launch_smem<64, 4>(A, grid, s);
    case 1: return launch_smem<128, 2>(A, grid, s);
    case 2: return capped ? launch_smem_capped<64, 8, 10>(A, grid, s) : launch_smem<64, 8>(A, grid, s);
    case 3: return launch_smem<128, 4>(A, grid, s);
    case 4: return launch_smem<256, 2>(A, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

int occupancy_variant_small(int v, bool capped) {
  switch (v) {
    case 0: return capped ? occupancy_smem_capped<64, 4, 12>() : occupancy_smem<64, 4>();
    case 1: return occupancy_smem<128, 2>();
    case 2: return capped ? occupancy_smem_capped<64, 8, 10>() : occupancy_smem<64, 8>();
    case 3: return occupancy_smem<128, 4>();
    case 4: return occupancy_smem<256, 2>();
    default: return -1;
  }
}

}  // namespace fjg
