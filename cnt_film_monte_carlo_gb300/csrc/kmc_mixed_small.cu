// kmc_mixed_small.cu -- mixed hop kernel variants with 128-thread blocks (0: 4, 1: 6, 2: 8
// resident blocks per SM).
#include "kmc_hop_mixed.cuh"

namespace kmc {

cudaError_t launch_hop_mixed_small(const HopArgs& a, int64_t n_steps, int variant, int grid_blocks, int single_film,
                                   unsigned long long* queue, cudaStream_t s) {
  switch (variant) {
    case 1: return launch_mixed_t<128, 6>(a, n_steps, grid_blocks, single_film, queue, s);
    case 2: return launch_mixed_t<128, 8>(a, n_steps, grid_blocks, single_film, queue, s);
    default: return launch_mixed_t<128, 4>(a, n_steps, grid_blocks, single_film, queue, s);
  }
}

int hop_mixed_blocks_per_sm_small(int variant, int64_t n_steps, int single_film) {
  switch (variant) {
    case 1: return blocks_per_sm_t<128, 6>(n_steps, single_film);
    case 2: return blocks_per_sm_t<128, 8>(n_steps, single_film);
    default: return blocks_per_sm_t<128, 4>(n_steps, single_film);
  }
}

}  // namespace kmc
