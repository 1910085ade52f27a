// Counter-based uniforms and fused Monte Carlo.
//
// The reference draws torch.rand([N, dim]) from the global generator
// (rng.py:120-125), scales it onto the domain (monte_carlo.py:102-106),
// evaluates the integrand and averages (monte_carlo.py:60-82).  Here the
// draws come from Philox4x32-10 keyed by the seed with an explicit block
// offset, so the fused kernel regenerates in registers exactly the values
// tq_uniform writes for the materialised path, and no [N, dim] buffer exists.

#include <type_traits>

#include "tq_common.cuh"

namespace tq {

template <typename T>
__global__ void __launch_bounds__(kBlock)
    uniform_kernel(uint64_t seed, uint64_t sid, uint64_t offset, int64_t numel, T* __restrict__ out) {
  constexpr int PB = Uniform<T>::per_block;
  const int64_t nblk = (numel + PB - 1) / PB;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblk;
       b += (int64_t)gridDim.x * blockDim.x) {
    const uint4 r = philox_block(seed, sid, offset + (uint64_t)b);
    const int64_t e0 = b * PB;
#pragma unroll
    for (int l = 0; l < PB; ++l)
      if (e0 + l < numel) out[e0 + l] = Uniform<T>::from(r, l);
  }
}

struct McArgs {
  int dim, family;
  int64_t n_points;
  uint64_t seed, sid, offset;
  const void* domain;
  const double* params;
  Acc* partials;
  unsigned* ticket;
  void* out;
  double* out64;
};

template <typename T, int FAM, int P>
__global__ void __launch_bounds__(kBlock) mc_fused_kernel(McArgs a) {
  __shared__ Family<T> fam;
  __shared__ T lo[kMaxDim], width[kMaxDim];
  __shared__ T volume;
  const T* dom = (const T*)a.domain;
  if (threadIdx.x == 0) {
    load_family<T>(fam, a.family, a.dim, a.params);
    T v = (T)1;
    for (int k = 0; k < a.dim; ++k) {
      lo[k] = dom[2 * k];
      width[k] = dom[2 * k + 1] - dom[2 * k];
      v = v * width[k];
    }
    volume = v;
  }
  __syncthreads();
  constexpr int PB = Uniform<T>::per_block;
  const int dim = a.dim;
  Acc acc{0.0, 0.0};
  F2 facc{0.f, 0.f};  // fp32: the strip sums as a double-float on the FP32 pipe
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * P; base < a.n_points;
       base += nthreads * P) {
    const int64_t end = min(base + P, a.n_points);
    T inner = T(0), comp = T(0);
    uint64_t cur_blk = ~0ull;
    uint4 r = make_uint4(0, 0, 0, 0);
    for (int64_t p = base; p < end; ++p) {
      T s = T(0);
      for (int k = 0; k < dim; ++k) {
        const uint64_t e = (uint64_t)p * dim + k;
        const uint64_t blk = e / PB;
        if (blk != cur_blk) {
          r = philox_block(a.seed, a.sid, a.offset + blk);
          cur_blk = blk;
        }
        const T u = Uniform<T>::from(r, (int)(e - blk * PB));
        // monte_carlo.py:106: uniform * domain_sizes + domain_starts
        const T x = u * width[k] + lo[k];
        const T g = fam_term<FAM, T>(fam, k, x);
        s = (k == 0) ? g : s + g;
      }
      const T f = fam_outer<FAM, T>(fam, s);
      // compensated strip sum in the working type
      const T t = inner + f;
      comp += (fabs(inner) >= fabs(f)) ? ((inner - t) + f) : ((f - t) + inner);
      inner = t;
    }
    if constexpr (std::is_same<T, float>::value)
      facc = f2_add(f2_add(facc, inner), comp);
    else
      acc_add(acc, (double)inner + (double)comp);
  }
  if constexpr (std::is_same<T, float>::value) acc_add(acc, f2_value(facc));
  acc = block_reduce<kBlock>(acc);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = acc;
  if (last_block_arrives(a.ticket)) {
    Acc t{0.0, 0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) acc_merge(t, a.partials[i]);
    t = block_reduce<kBlock>(t);
    if (threadIdx.x == 0) {
      const double v = (double)volume * (t.s + t.c) / (double)a.n_points;
      if (a.out) *(T*)a.out = (T)v;
      if (a.out64) *a.out64 = v;
      *a.ticket = 0u;
    }
  }
}

}  // namespace tq

using namespace tq;

extern "C" int tq_uniform(int dtype, uint64_t seed, uint64_t stream_id, uint64_t offset,
                          int64_t numel, void* out, void* stream) {
  if (!valid_dtype(dtype)) return TQ_ERR_DTYPE;
  if (numel < 0 || (!out && numel > 0)) return TQ_ERR_ARG;
  if (numel == 0) return TQ_OK;
  const int64_t nblk = (numel + (dtype == TQ_F64 ? 1 : 3)) / (dtype == TQ_F64 ? 2 : 4);
  int64_t grid = (nblk + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (grid > cap) grid = cap;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TQ_F64)
    uniform_kernel<double><<<(unsigned)grid, kBlock, 0, s>>>(seed, stream_id, offset, numel,
                                                             (double*)out);
  else
    uniform_kernel<float><<<(unsigned)grid, kBlock, 0, s>>>(seed, stream_id, offset, numel,
                                                            (float*)out);
  return launch_status();
}

static constexpr int kStripMC = 8;

static int64_t mc_blocks(int64_t n) {
  const int64_t need = (n + (int64_t)kBlock * kStripMC - 1) / ((int64_t)kBlock * kStripMC);
  const int64_t cap = (int64_t)sm_count() * 8;
  return need < 1 ? 1 : (need < cap ? need : cap);
}

extern "C" size_t tq_mc_fused_workspace_size(int dim, int64_t n_points) {
  (void)dim;
  return reduce_ws_bytes(mc_blocks(n_points));
}

extern "C" int tq_mc_fused(int dtype, int dim, int64_t n_points, const void* domain, int family,
                           const double* params, uint64_t seed, uint64_t stream_id,
                           uint64_t offset, void* out, double* out64, void* workspace,
                           size_t workspace_bytes, void* stream) {
  if (!valid_dtype(dtype)) return TQ_ERR_DTYPE;
  if (dim < 1 || dim > kMaxDim) return TQ_ERR_DIM;
  if (n_points < 1 || !domain || !params || !workspace || (!out && !out64)) return TQ_ERR_ARG;
  if (n_points > (int64_t(1) << 60) / dim) return TQ_ERR_TOO_LARGE;
  const int64_t blocks = mc_blocks(n_points);
  if (workspace_bytes < reduce_ws_bytes(blocks)) return TQ_ERR_WORKSPACE;
  McArgs a;
  a.dim = dim;
  a.family = family;
  a.n_points = n_points;
  a.seed = seed;
  a.sid = stream_id;
  a.offset = offset;
  a.domain = domain;
  a.params = params;
  a.ticket = (unsigned*)workspace;
  a.partials = (Acc*)((char*)workspace + 256);
  a.out = out;
  a.out64 = out64;
  cudaStream_t s = (cudaStream_t)stream;
  TQ_DISPATCH_FAMILY(family, FAM, {
    if (dtype == TQ_F64)
      mc_fused_kernel<double, FAM, kStripMC><<<(unsigned)blocks, kBlock, 0, s>>>(a);
    else
      mc_fused_kernel<float, FAM, kStripMC><<<(unsigned)blocks, kBlock, 0, s>>>(a);
  });
  return launch_status();
}
