// kmc_mixed_large.cu -- mixed hop kernel variants with larger blocks (3: 256 threads x 3
// resident blocks per SM, 4: 768 threads x 1, 5: 1024 threads x 1).
#include "kmc_hop_mixed.cuh"

namespace kmc {

cudaError_t launch_hop_mixed_large(const HopArgs& a, int64_t n_steps, int variant, int grid_blocks, int single_film,
                                   unsigned long long* queue, cudaStream_t s) {
  if (variant == 4) return launch_mixed_t<768, 1>(a, n_steps, grid_blocks, single_film, queue, s);
  if (variant == 5) return launch_mixed_t<1024, 1>(a, n_steps, grid_blocks, single_film, queue, s);
  return launch_mixed_t<256, 3>(a, n_steps, grid_blocks, single_film, queue, s);
}

int hop_mixed_blocks_per_sm_large(int variant, int64_t n_steps, int single_film) {
  if (variant == 4) return blocks_per_sm_t<768, 1>(n_steps, single_film);
  if (variant == 5) return blocks_per_sm_t<1024, 1>(n_steps, single_film);
  return blocks_per_sm_t<256, 3>(n_steps, single_film);
}

}  // namespace kmc
