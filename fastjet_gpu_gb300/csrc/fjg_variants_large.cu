// Shared-memory kernel variants of capacity 1024, 2048 and 4096 particles.
#include "fjg_variants.cuh"

namespace fjg {

static_assert(sizeof(SmemLayout<256, 8>) + 1024 <= 233472 / 3, "capacity 2048 at 256 threads: three CTAs per SM");
static_assert(sizeof(SmemLayout<128, 8>) + 1024 <= 233472 / 5, "capacity 1024 at 128 threads: five CTAs per SM");
static_assert(sizeof(SmemLayout<512, 4>) <= 232448, "capacity 2048 at 512 threads: one CTA per SM");
static_assert(sizeof(SmemLayout<512, 8>) <= 232448, "capacity 4096: one CTA per SM");
static_assert(sizeof(SmemLayout<256, 16>) <= 232448, "capacity 4096: one CTA per SM");

cudaError_t launch_variant_large(int v, const BatchArgs& A, int grid, bool capped, cudaStream_t s) {
  switch (v) {
    case 5: return capped ? launch_smem_capped<128, 8, 5>(A, grid, s) : launch_smem<128, 8>(A, grid, s);
    case 6: return launch_smem<256, 4>(A, grid, s);
    case 7: return capped ? launch_smem_capped<256, 8, 3>(A, grid, s) : launch_smem<256, 8>(A, grid, s);
    case 8: return launch_smem<512, 4>(A, grid, s);
    case 9: return launch_smem<512, 8>(A, grid, s);
    case 10: return launch_smem<256, 16>(A, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

int occupancy_variant_large(int v, bool capped) {
  switch (v) {
    case 5: return capped ? occupancy_smem_capped<128, 8, 5>() : occupancy_smem<128, 8>();
    case 6: return occupancy_smem<256, 4>();
    case 7: return capped ? occupancy_smem_capped<256, 8, 3>() : occupancy_smem<256, 8>();
    case 8: return occupancy_smem<512, 4>();
    case 9: return occupancy_smem<512, 8>();
    case 10: return occupancy_smem<256, 16>();
    default: return -1;
  }
}

}  // namespace fjg
