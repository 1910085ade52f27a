// Grid geometry shared by the fused grid rules and their adjoint: per-
// dimension nodes and 1-D weights of the tensor-product rules.
#pragma once

#include "tq_common.cuh"

namespace tq {

// Per-dimension geometry of the grid, computed once per CTA from the domain.
template <typename T>
struct Geo {
  T a[kMaxDim], b[kMaxDim], step[kMaxDim];
  // weight scale of a dimension: NC rules h * (1/2 | 1/3 | 1/22.5), Gauss
  // 0.5 * (b - a); both rounded as the reference rounds them, then widened.
  double wscale[kMaxDim];
  double half[kMaxDim], mid[kMaxDim];  // Gauss node map (b-a)/2 * r + (a+b)/2
};

// Integer part of the Newton-Cotes weights (exact in any float type).
__device__ __forceinline__ int nc_int(int rule, int64_t i, int64_t n) {
  if (rule == TQ_RULE_TRAPEZOID) return (i == 0 || i == n - 1) ? 1 : 2;
  if (rule == TQ_RULE_SIMPSON) return (i == 0 || i == n - 1) ? 1 : ((i & 1) ? 4 : 2);
  if (i == 0 || i == n - 1) return 7;
  const int m = (int)(i & 3);
  return (m & 1) ? 32 : (m == 2 ? 12 : 14);
}
__host__ __device__ __forceinline__ double nc_den(int rule) {
  return rule == TQ_RULE_TRAPEZOID ? 2.0 : (rule == TQ_RULE_SIMPSON ? 3.0 : 22.5);
}

// D = domain type.  Fills g from domain[dim][2] (device, read by thread 0).
template <typename T, typename D>
__device__ void geo_setup(Geo<T>& g, int rule, int dim, int64_t n, const D* __restrict__ dom) {
  for (int k = 0; k < dim; ++k) {
    const D a = dom[2 * k], b = dom[2 * k + 1];
    g.a[k] = (T)a;
    g.b[k] = (T)b;
    if (rule == TQ_RULE_GAUSS) {
      // gaussian.py:159-162 in the domain type, then fp64 with the roots
      const D hw = (D)(b - a) / (D)2;
      const D md = (D)(a + b) / (D)2;
      g.half[k] = (double)hw;
      g.mid[k] = (double)md;
      g.wscale[k] = (double)((D)0.5 * (D)(b - a));  // gaussian.py:141-143
      g.step[k] = (T)0;
    } else if (rule == TQ_RULE_MC) {
      g.step[k] = (T)0;
      g.wscale[k] = 1.0;
    } else {
      const T ta = (T)a, tb = (T)b;
      const T st = (tb - ta) / (T)(n - 1);
      g.step[k] = st;
      // h = grid[1] - grid[0] in the working type (integration_grid.py:90-93)
      const T h = linspace_node<T>(ta, tb, st, n, 1) - linspace_node<T>(ta, tb, st, n, 0);
      g.wscale[k] = (double)h / nc_den(rule);
      g.half[k] = g.mid[k] = 0.0;
    }
  }
}

template <typename T, bool GL>
__device__ __forceinline__ T node_at(const Geo<T>& g, int k, int64_t n, int64_t i,
                                     const double* __restrict__ gl_nodes) {
  if (GL) return (T)__dadd_rn(__dmul_rn(g.half[k], __ldg(gl_nodes + i)), g.mid[k]);
  return linspace_node<T>(g.a[k], g.b[k], g.step[k], n, i);
}
// Unscaled 1-D weight (integer NC coefficient or Gauss weight).
template <bool GL>
__device__ __forceinline__ double wunit_at(int rule, int64_t n, int64_t i,
                                           const double* __restrict__ gl_w) {
  if (GL) return __ldg(gl_w + i);
  return (double)nc_int(rule, i, n);
}

// Integer Newton-Cotes coefficient of node j, the rule fixed at compile time.
template <int RULE>
__device__ __forceinline__ int nc_int_t(int j, int n) {
  if (j == 0 || j == n - 1) return RULE == TQ_RULE_TRAPEZOID ? 1 : (RULE == TQ_RULE_SIMPSON ? 1 : 7);
  if (RULE == TQ_RULE_TRAPEZOID) return 2;
  if (RULE == TQ_RULE_SIMPSON) return (j & 1) ? 4 : 2;
  const int m = j & 3;
  return (m & 1) ? 32 : (m == 2 ? 12 : 14);
}

}  // namespace tq
