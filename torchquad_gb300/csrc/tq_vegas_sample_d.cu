// The fused VEGAS sampler for fp32 iterations specialised on the dimension
// (1..8): a separate translation unit so that it compiles in parallel with
// the rest of the VEGAS code.

#include "tq_vegas_sample.cuh"

namespace tq {

template <int FAM, int D>
static int launch_dims(const SampleArgs& a, unsigned grid, size_t smem, cudaStream_t s) {
  auto kfn = vegas_sample_kernel<float, FAM, false, D>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_cuda_error(e);
  }
  kfn<<<grid, kTile, smem, s>>>(a);
  return launch_status();
}

template <int FAM>
static int launch_fam(const SampleArgs& a, int dim, unsigned grid, size_t smem, cudaStream_t s) {
  switch (dim) {
    case 1: return launch_dims<FAM, 1>(a, grid, smem, s);
    case 2: return launch_dims<FAM, 2>(a, grid, smem, s);
    case 3: return launch_dims<FAM, 3>(a, grid, smem, s);
    case 4: return launch_dims<FAM, 4>(a, grid, smem, s);
    case 5: return launch_dims<FAM, 5>(a, grid, smem, s);
    case 6: return launch_dims<FAM, 6>(a, grid, smem, s);
    case 7: return launch_dims<FAM, 7>(a, grid, smem, s);
    case 8: return launch_dims<FAM, 8>(a, grid, smem, s);
    default: return TQ_ERR_ARG;
  }
}

int launch_sample_f32_dims(const SampleArgs& a, int family, int dim, unsigned grid, size_t smem,
                           cudaStream_t s) {
  int rc = TQ_ERR_ARG;
  TQ_DISPATCH_FAMILY(family, FAM, { rc = launch_fam<FAM>(a, dim, grid, smem, s); });
  return rc;
}

}  // namespace tq
