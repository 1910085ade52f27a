// Batched tensor-product rules: many integrals of different rule, dimension,
// points per dimension and domain in one persistent launch.
//
// Each integral i is cut into tiles of `tile_pts` consecutive flat node
// indices; tile_start[i] is the exclusive prefix of the tile counts.  CTAs
// stride over the flat tile list, find a tile's integral by binary search in
// tile_start, set the integral's geometry up in shared memory and sum the
// tile's nodes with the same row-segment walk as the single fused rule
// (strips of P nodes per thread, last dimension innermost).  Each tile's
// compensated partial goes to partials[tile]; a second kernel reduces every
// integral's tiles in tile order (deterministic, no atomics).
//
// The reference has no batched form: a batch is a loop of per-call
// GridIntegrator.integrate (grid_integrator.py:32-55).

#include "tq_grid_common.cuh"

namespace tq {

struct BatchDesc {
  int32_t rule, dim;
  int64_t n, total;
  int64_t par_off;  // into params (fp64, 2 + 2*dim values)
  int64_t dom_off;  // into domains (dtype, 2*dim values)
  int64_t gl_off;   // into gl_nodes / gl_weights (Gauss only)
};

struct BatchArgs {
  const BatchDesc* desc;
  const int64_t* tile_start;  // [n_int + 1]
  int64_t n_int, n_tiles, tile_pts;
  const double* params;
  const void* domains;
  const double* gl_nodes;
  const double* gl_weights;
  int family;
  Acc* partials;  // [n_tiles]
};

template <typename T, int FAM, int P>
__global__ void __launch_bounds__(256) batch_grid_kernel(BatchArgs a) {
  __shared__ Geo<T> g;
  __shared__ Family<T> fam;
  __shared__ uint64_t rstride[kMaxDim];
  __shared__ BatchDesc d;
  __shared__ int64_t tile0;
  for (int64_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
    if (threadIdx.x == 0) {
      int64_t lo = 0, hi = a.n_int;  // largest i with tile_start[i] <= tile
      while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (a.tile_start[mid] <= tile) lo = mid;
        else hi = mid;
      }
      d = a.desc[lo];
      tile0 = a.tile_start[lo];
      geo_setup<T, T>(g, d.rule, d.dim, d.n, (const T*)a.domains + d.dom_off);
      load_family<T>(fam, a.family, d.dim, a.params + d.par_off);
      uint64_t st = 1;
      for (int k = d.dim - 2; k >= 0; --k) {
        rstride[k] = st;
        st *= (uint64_t)d.n;
      }
    }
    __syncthreads();
    const int dim = d.dim, rule = d.rule, last = dim - 1;
    const int64_t n = d.n;
    const int n32 = (int)n;
    const bool gl = rule == TQ_RULE_GAUSS;
    const double* gln = a.gl_nodes + d.gl_off;
    const double* glw = a.gl_weights + d.gl_off;
    const int64_t begin = (tile - tile0) * a.tile_pts;
    const int64_t end = min(d.total, begin + a.tile_pts);
    const double wlast = g.wscale[last];
    const T a_l = g.a[last], b_l = g.b[last], st_l = g.step[last];
    const int half = n32 / 2;
    Acc acc{0.0, 0.0};
    for (int64_t base = begin + (int64_t)threadIdx.x * P; base < end;
         base += (int64_t)blockDim.x * P) {
      uint64_t row = (uint64_t)base / (uint64_t)n;
      int jl = (int)(base - (int64_t)row * n);
      int64_t left = min((int64_t)P, end - base);
      while (left > 0) {
        T s_outer = T(0);
        double w_outer = 1.0;
        for (int k = 0; k < dim - 1; ++k) {
          const int64_t digit = (int64_t)((row / rstride[k]) % (uint64_t)n);
          const T x = gl ? (T)__dadd_rn(__dmul_rn(g.half[k], __ldg(gln + digit)), g.mid[k])
                         : linspace_node<T>(g.a[k], g.b[k], g.step[k], n, digit);
          const T t = fam_term<FAM, T>(fam, k, x);
          s_outer = (k == 0) ? t : s_outer + t;
          w_outer *= g.wscale[k] * (gl ? __ldg(glw + digit) : (double)nc_int(rule, digit, n));
        }
        const int seg_end = (int)min((int64_t)n32, (int64_t)jl + left);
        T sum = T(0), comp = T(0);
        for (int j = jl; j < seg_end; ++j) {
          T x;
          if (gl)
            x = (T)__dadd_rn(__dmul_rn(g.half[last], __ldg(gln + j)), g.mid[last]);
          else
            x = (j < half) ? fma(st_l, (T)j, a_l) : fma(-st_l, (T)(n32 - 1 - j), b_l);
          const T f = fam_outer<FAM, T>(fam, s_outer + fam_term<FAM, T>(fam, last, x));
          const T wj = gl ? (T)__ldg(glw + j) : (T)nc_int(rule, j, n);
          // Kahan in the working type within the segment
          const T y = wj * f - comp;
          const T tt = sum + y;
          comp = (tt - sum) - y;
          sum = tt;
        }
        acc_add(acc, ((double)sum - (double)comp) * (w_outer * wlast));
        left -= seg_end - jl;
        jl = 0;
        ++row;
      }
    }
    acc = block_reduce<256>(acc);
    if (threadIdx.x == 0) a.partials[tile] = acc;
    __syncthreads();
  }
}

// One warp per integral: compensated sum of its tiles in tile order.
__global__ void batch_finalize_kernel(const int64_t* tile_start, int64_t n_int, const Acc* partials,
                                      void* out, int out_dtype) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n_int) return;
  const int64_t t0 = tile_start[w], t1 = tile_start[w + 1];
  Acc a{0.0, 0.0};
  for (int64_t t = t0 + lane; t < t1; t += 32) acc_merge(a, partials[t]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc_merge(a, acc_shfl_down(a, o));
  if (lane == 0) {
    const double v = a.s + a.c;
    if (out_dtype == TQ_F64)
      ((double*)out)[w] = v;
    else
      ((float*)out)[w] = (float)v;
  }
}

}  // namespace tq

using namespace tq;

extern "C" int tq_batch_grid(int dtype, int64_t n_integrals, const void* descs,
                             const int64_t* tile_start, int64_t n_tiles, int64_t tile_points,
                             const double* params, const void* domains, const double* gl_nodes,
                             const double* gl_weights, int family, int block, int strip,
                             int grid_blocks, void* out, int out_dtype, void* workspace,
                             size_t workspace_bytes, void* stream) {
  if (!valid_dtype(dtype) || !valid_dtype(out_dtype)) return TQ_ERR_DTYPE;
  if (n_integrals < 1 || n_tiles < 1 || tile_points < 1 || !descs || !tile_start || !params ||
      !domains || !out || !workspace)
    return TQ_ERR_ARG;
  if (block != 128 && block != 256) return TQ_ERR_ARG;
  if (strip != 4 && strip != 16) return TQ_ERR_ARG;
  if (workspace_bytes < (size_t)n_tiles * sizeof(Acc)) return TQ_ERR_WORKSPACE;
  BatchArgs a;
  a.desc = (const BatchDesc*)descs;
  a.tile_start = tile_start;
  a.n_int = n_integrals;
  a.n_tiles = n_tiles;
  a.tile_pts = tile_points;
  a.params = params;
  a.domains = domains;
  a.gl_nodes = gl_nodes ? gl_nodes : params;  // unused unless an integral is Gauss
  a.gl_weights = gl_weights ? gl_weights : params;
  a.family = family;
  a.partials = (Acc*)workspace;
  int64_t grid = grid_blocks > 0 ? grid_blocks : (int64_t)sm_count() * 8;
  if (grid > n_tiles) grid = n_tiles;
  cudaStream_t s = (cudaStream_t)stream;
#define TQ_BATCH(T, PV) batch_grid_kernel<T, FAM, PV><<<(unsigned)grid, block, 0, s>>>(a)
  TQ_DISPATCH_FAMILY(family, FAM, {
    if (dtype == TQ_F64) {
      if (strip == 4) TQ_BATCH(double, 4);
      else TQ_BATCH(double, 16);
    } else {
      if (strip == 4) TQ_BATCH(float, 4);
      else TQ_BATCH(float, 16);
    }
  });
#undef TQ_BATCH
  int e = launch_status();
  if (e != TQ_OK) return e;
  const unsigned fb = (unsigned)((n_integrals * 32 + 255) / 256);
  batch_finalize_kernel<<<fb, 256, 0, s>>>(tile_start, n_integrals, (const Acc*)workspace, out,
                                           out_dtype);
  return launch_status();
}
