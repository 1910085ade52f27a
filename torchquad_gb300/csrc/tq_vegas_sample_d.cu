// The fused VEGAS sampler for fp32 states specialised on the dimension
// (1..8), for iterations and warm-up: a separate translation unit so that it
// compiles in parallel with the rest of the VEGAS code.

#include "tq_vegas_sample.cuh"

namespace tq {

template <int FAM, bool WARM, int D>
static int launch_dims(const SampleArgs& a, unsigned grid, size_t smem, cudaStream_t s) {
  auto kfn = vegas_sample_kernel<float, FAM, WARM, D>;
  const int rc = opt_in_smem(kfn, smem);
  if (rc != TQ_OK) return rc;
  kfn<<<grid, kTile, smem, s>>>(a);
  return launch_status();
}

template <int FAM, bool WARM>
static int launch_fam(const SampleArgs& a, int dim, unsigned grid, size_t smem, cudaStream_t s) {
  switch (dim) {
    case 1: return launch_dims<FAM, WARM, 1>(a, grid, smem, s);
    case 2: return launch_dims<FAM, WARM, 2>(a, grid, smem, s);
    case 3: return launch_dims<FAM, WARM, 3>(a, grid, smem, s);
    case 4: return launch_dims<FAM, WARM, 4>(a, grid, smem, s);
    case 5: return launch_dims<FAM, WARM, 5>(a, grid, smem, s);
    case 6: return launch_dims<FAM, WARM, 6>(a, grid, smem, s);
    case 7: return launch_dims<FAM, WARM, 7>(a, grid, smem, s);
    case 8: return launch_dims<FAM, WARM, 8>(a, grid, smem, s);
    default: return TQ_ERR_ARG;
  }
}

int launch_sample_f32_dims(const SampleArgs& a, int family, int dim, bool warm, unsigned grid,
                           size_t smem, cudaStream_t s) {
  int rc = TQ_ERR_ARG;
  if (warm) {
    TQ_DISPATCH_FAMILY(family, FAM, { rc = launch_fam<FAM, true>(a, dim, grid, smem, s); });
  } else {
    TQ_DISPATCH_FAMILY(family, FAM, { rc = launch_fam<FAM, false>(a, dim, grid, smem, s); });
  }
  return rc;
}

}  // namespace tq
