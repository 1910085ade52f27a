// Peak probe: a long chain of independent fp32 FMAs per thread, used by the
// benchmark to measure the FP32 FMA roofline of the device it runs on.
#include "tq_common.cuh"

namespace tq {

__global__ void __launch_bounds__(kBlock) fma_probe_kernel(int64_t iters, float seed, float* out) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + (float)(threadIdx.x + i);
  const float m = 0.999999f, c = 1e-7f;
  for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], m, c);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == 123.456f) out[0] = s;  // keeps the chain live; practically never stores
}

// The same chain in fp64: the FP64-pipe peak (GB300 runs FP64 at a small
// fraction of its FP32 rate).
__global__ void __launch_bounds__(kBlock) dfma_probe_kernel(int64_t iters, double seed, double* out) {
  double a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + (double)(threadIdx.x + i);
  const double m = 0.999999, c = 1e-7;
  for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = fma(a[i], m, c);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == 123.456) out[0] = s;
}

}  // namespace tq

// Launches sm_count * blocks_per_sm CTAs of 256 threads, each thread doing
// iters * 128 FMAs (2 flops each); returns the number of flops launched in
// *flops.  The caller times the launch.
extern "C" int tq_fp32_fma_probe(int64_t iters, int blocks_per_sm, float* out, double* flops,
                                 void* stream) {
  if (iters < 1 || blocks_per_sm < 1 || !out || !flops) return TQ_ERR_ARG;
  const int grid = tq::sm_count() * blocks_per_sm;
  tq::fma_probe_kernel<<<grid, tq::kBlock, 0, (cudaStream_t)stream>>>(iters, 1.0f, out);
  *flops = 2.0 * 128.0 * (double)iters * (double)grid * tq::kBlock;
  return tq::launch_status();
}

// tq_fp32_fma_probe with fp64 fused multiply-adds (out: one double).
extern "C" int tq_fp64_fma_probe(int64_t iters, int blocks_per_sm, double* out, double* flops,
                                 void* stream) {
  if (iters < 1 || blocks_per_sm < 1 || !out || !flops) return TQ_ERR_ARG;
  const int grid = tq::sm_count() * blocks_per_sm;
  tq::dfma_probe_kernel<<<grid, tq::kBlock, 0, (cudaStream_t)stream>>>(iters, 1.0, out);
  *flops = 2.0 * 128.0 * (double)iters * (double)grid * tq::kBlock;
  return tq::launch_status();
}
