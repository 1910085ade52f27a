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

// ------------------------------- fp64 rows of equally spaced nodes by recurrence
// Along a grid row of a Newton-Cotes rule the last coordinate steps by h,
// so each built-in family's value at the next node follows from the
// current one by a few multiplies instead of an exp / cos (one FP64 warp
// instruction holds a GB300 sub-partition's FP64 unit for about 64 cycles):
//   exp sum      f_{j+1} = f_j q,                 q = exp(a h)
//   Gaussian     f_{j+1} = f_j r_j,  r_{j+1} = r_j q,  q = exp(-2 a h^2),
//                r_j = exp(-a h (2 (x_j - u) + h))
//   oscillatory  (cos, sin) of the angle rotated by a h each node
//   sum of sines sin(a x) rotated likewise.
// A segment starts from a direct evaluation at its first node, so rounding
// accumulates over at most a segment's length (16-32 nodes): a few ulps
// per node value, far inside the grid rules' 1e-12 tolerance.
struct RecurConst {
  double q, cd, sd;  // exp-family factor; cosine and sine of the angle step
};

template <int FAM>
__device__ __forceinline__ RecurConst recur_const(const Family<double>& fam, int last, double h) {
  RecurConst rc{1.0, 1.0, 0.0};
  const double a = fam.a[last];
  if (FAM == TQ_FN_EXP_SUM) {
    rc.q = exp(a * h);
  } else if (FAM == TQ_FN_GAUSSIAN) {
    rc.q = exp(-2.0 * a * h * h);
  } else {
    sincos(a * h, &rc.sd, &rc.cd);
  }
  return rc;
}

// Newton-Cotes integer coefficient of node j as a float, the rule chosen at
// run time, without an integer-to-float conversion.
__device__ __forceinline__ float nc_coef_f(int rule, int j, int n) {
  if (j == 0 || j == n - 1) return rule == TQ_RULE_BOOLE ? 7.f : 1.f;
  if (rule == TQ_RULE_TRAPEZOID) return 2.f;
  if (rule == TQ_RULE_SIMPSON) return (j & 1) ? 4.f : 2.f;
  const int m = j & 3;
  return (m & 1) ? 32.f : (m == 2 ? 12.f : 14.f);
}

// Newton-Cotes integer coefficient of node j as a double, without an
// integer-to-double conversion.
template <int RULE>
__device__ __forceinline__ double nc_coef_d(int j, int n) {
  if (j == 0 || j == n - 1) return RULE == TQ_RULE_TRAPEZOID ? 1.0 : (RULE == TQ_RULE_SIMPSON ? 1.0 : 7.0);
  if (RULE == TQ_RULE_TRAPEZOID) return 2.0;
  if (RULE == TQ_RULE_SIMPSON) return (j & 1) ? 4.0 : 2.0;
  const int m = j & 3;
  return (m & 1) ? 32.0 : (m == 2 ? 12.0 : 14.0);
}

// sum_{j0 <= j < j1} coef_j f(s + g(x_j)), x_j0 = x0, x_{j+1} = x_j + h, for
// a row of n nodes (fp64, Newton-Cotes rules), into *out.  Returns false
// (nothing computed) where a recurrence could leave the range of doubles,
// and the caller then evaluates the nodes directly: the exponent must stay
// in [-600, 600] over the segment (linear in j for the exp sum, so its ends
// bound it; concave for a Gaussian with a >= 0, so its ends bound it from
// below and its peak value -s from above) and change by at most 690 from
// one node to the next (for the Gaussian that change is linear in j: its
// first and last steps bound it).
template <int FAM, int RULE>
__device__ bool recur_seg(const Family<double>& fam, const RecurConst& rc, int last, double s, double x0,
                          double x1, double h, int j0, int j1, int n, double* out) {
  const double a = fam.a[last];
  double acc = 0.0;
  if (FAM == TQ_FN_EXP_SUM) {
    const double e0 = s + a * x0 + fam.b, e1 = s + a * x1 + fam.b;
    if (!(fabs(e0) <= 600.0 && fabs(e1) <= 600.0 && fabs(a * h) <= 690.0)) return false;
    double f = fam.c * exp(e0);
    for (int j = j0; j < j1; ++j) {
      acc = fma(nc_coef_d<RULE>(j, n), f, acc);
      f *= rc.q;
    }
  } else if (FAM == TQ_FN_GAUSSIAN) {
    const double d0 = x0 - fam.u[last], d1 = x1 - fam.u[last];
    const double e0 = -(s + a * (d0 * d0)), e1 = -(s + a * (d1 * d1));
    if (!(a >= 0.0 && -s <= 600.0 && fabs(e0) <= 600.0 && fabs(e1) <= 600.0 &&
          fabs(a * h * (2.0 * d0 + h)) <= 690.0 && fabs(a * h * (2.0 * d1 - h)) <= 690.0 && rc.q > 1e-300))
      return false;
    double f = fam.c * exp(e0);
    double r = exp(-a * h * (2.0 * d0 + h));
    for (int j = j0; j < j1; ++j) {
      acc = fma(nc_coef_d<RULE>(j, n), f, acc);
      f *= r;
      r *= rc.q;
    }
  } else {
    double sn, cs;  // oscillatory: angle 2 pi b + s + a x; sum of sines: a x
    if (FAM == TQ_FN_OSCILLATORY)
      sincos(2.0 * CUDART_PI * fam.b + s + a * x0, &sn, &cs);
    else
      sincos(a * x0, &sn, &cs);
    for (int j = j0; j < j1; ++j) {
      const double v = FAM == TQ_FN_OSCILLATORY ? cs : s + sn;
      acc = fma(nc_coef_d<RULE>(j, n), v, acc);
      const double c2 = fma(cs, rc.cd, -(sn * rc.sd));
      sn = fma(sn, rc.cd, cs * rc.sd);
      cs = c2;
    }
    acc *= fam.c;
  }
  *out = acc;
  return true;
}

// recur_seg with the rule chosen at run time.
template <int FAM>
__device__ __forceinline__ bool recur_seg_rule(int rule, const Family<double>& fam, const RecurConst& rc, int last,
                                               double s, double x0, double x1, double h, int j0, int j1, int n,
                                               double* out) {
  if (rule == TQ_RULE_TRAPEZOID)
    return recur_seg<FAM, TQ_RULE_TRAPEZOID>(fam, rc, last, s, x0, x1, h, j0, j1, n, out);
  if (rule == TQ_RULE_SIMPSON) return recur_seg<FAM, TQ_RULE_SIMPSON>(fam, rc, last, s, x0, x1, h, j0, j1, n, out);
  return recur_seg<FAM, TQ_RULE_BOOLE>(fam, rc, last, s, x0, x1, h, j0, j1, n, out);
}

// ---------------------------------------------- fp64 inner-dimension tables
// The built-in families are functions of a separable sum s + t, where s
// gathers the outer dimensions of a grid row and t = g_last(x_j) the node's
// last coordinate.  For fp64 grids the node value is formed from a per-row
// factor and a per-node table entry instead of one fp64 exp/cos per node
// (on GB300 an FP64 warp instruction occupies the FP64 unit for ~64 cycles):
//   ExpSum   c exp(s + b + t)      = [c exp(s + b)] * exp(t)
//   Gaussian c exp(-(s + t))       = [c exp(-s)]    * exp(-t)
//   Oscill.  c cos(2 pi b + s + t) = [c cos p] cos t - [c sin p] sin t,  p = 2 pi b + s
//   SumSin   c (s + sin(a x))      = c * (s + t')
// Every node is still evaluated (a product of two normal numbers is correct
// to 2 ulp).  Rows whose factor is not a normal number, and tables with an
// entry that is not, take the direct formula.
constexpr int kTabMax = 1024;  // last-dimension nodes a table holds

// The node entries carry the node's weight: a node then costs one fused
// multiply-add into the row sum (two for the oscillatory and sum-of-sines
// families).
struct InnerTab {
  double w[kTabMax];   // unscaled 1-D weight of the last dimension
  double t1[kTabMax];  // w exp(t), w exp(-t), w cos(t) or w sin(a x)
  double t2[kTabMax];  // w sin(t) (oscillatory)
};

__device__ __forceinline__ bool normal_factor(double v) {
  return isfinite(v) && fabs(v) >= 2.2250738585072014e-308;
}

// Builds the table for nodes 0..n-1 of the last dimension (all threads of
// the CTA); returns, in every thread, whether all entries are usable.
template <int FAM>
__device__ bool build_inner_tab(InnerTab& tb, const Geo<double>& g, const Family<double>& fam,
                                int last, int n, bool gl, int rule,
                                const double* __restrict__ gl_nodes,
                                const double* __restrict__ gl_w) {
  int bad = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double x = gl ? __dadd_rn(__dmul_rn(g.half[last], __ldg(gl_nodes + j)), g.mid[last])
                        : linspace_node<double>(g.a[last], g.b[last], g.step[last], n, j);
    const double w = gl ? __ldg(gl_w + j) : (double)nc_int(rule, j, n);
    tb.w[j] = w;
    const double t = fam_term<FAM, double>(fam, last, x);
    if (FAM == TQ_FN_OSCILLATORY) {
      double sn, cs;
      sincos(t, &sn, &cs);
      tb.t1[j] = w * cs;
      tb.t2[j] = w * sn;
    } else if (FAM == TQ_FN_SUM_SIN) {
      tb.t1[j] = w * t;
    } else {
      const double e = exp(FAM == TQ_FN_GAUSSIAN ? -t : t);
      tb.t1[j] = w * e;
      bad |= !normal_factor(e) || !normal_factor(w * e);
    }
  }
  return !__syncthreads_or(bad);
}

// The row's factors for the separable sum s of its outer dimensions.
struct RowFactor {
  double r1, r2;
  bool ok;
};
template <int FAM>
__device__ __forceinline__ RowFactor row_factor(const Family<double>& fam, double s) {
  RowFactor f;
  if (FAM == TQ_FN_OSCILLATORY) {
    double sn, cs;
    sincos(2.0 * CUDART_PI * fam.b + s, &sn, &cs);
    f.r1 = fam.c * cs;
    f.r2 = fam.c * sn;
    f.ok = true;
  } else if (FAM == TQ_FN_SUM_SIN) {
    f.r1 = s;
    f.r2 = fam.c;
    f.ok = true;
  } else {
    f.r1 = fam.c * exp(FAM == TQ_FN_GAUSSIAN ? -s : s + fam.b);
    f.r2 = 0.0;
    f.ok = normal_factor(f.r1) || (f.r1 == 0.0 && fam.c == 0.0);
  }
  return f;
}
// seg + w_j f(node j) of a row from the row's factors and the node's
// weighted table entries (one or two fused multiply-adds).
template <int FAM>
__device__ __forceinline__ double tab_accum(double seg, double r1, double r2, const InnerTab& tb, int j) {
  if (FAM == TQ_FN_OSCILLATORY) return fma(-r2, tb.t2[j], fma(r1, tb.t1[j], seg));
  if (FAM == TQ_FN_SUM_SIN) return fma(r2, fma(r1, tb.w[j], tb.t1[j]), seg);
  return fma(r1, tb.t1[j], seg);
}

// Weighted sum over the nodes [begin, end) of an fp64 grid whose last
// dimension has a usable table.  The CTA first forms the outer state of
// each grid row in the range (a chunk of up to kRowChunk rows at a time:
// digits by multiply-high division, separable sum, outer weight and row
// factor; one outer-function evaluation per row, one thread per row) in
// shared memory; then its threads walk strips of kTabP consecutive nodes:
// value = row factor x table entry, one fused multiply-add per node into
// the row-segment sum, one per row segment into the strip sum, and a
// compensated add per strip.  Returns the thread's compensated partial.
constexpr int kRowChunk = 512;
constexpr int kTabP = 32;

struct RowTab {
  double p[kRowChunk], q[kRowChunk], w[kRowChunk], s[kRowChunk];
  int ok[kRowChunk];
};

template <int FAM>
__device__ Acc tab_rows_sum(const Geo<double>& g, const Family<double>& fam, const InnerTab& tab, RowTab& rt,
                            int dim, int rule, bool gl, int64_t n, const FastDiv& fdn,
                            const double* __restrict__ gl_nodes, const double* __restrict__ gl_w, int64_t begin,
                            int64_t end) {
  const int last = dim - 1;
  const int n32 = (int)n;
  const int64_t row_first = begin / n, row_last = (end - 1) / n;
  const bool small = end <= (int64_t)0xffffffffll;
  const double wlast = g.wscale[last];
  Acc acc{0.0, 0.0};
  for (int64_t rc = row_first; rc <= row_last; rc += kRowChunk) {
    const int nr = (int)min((int64_t)kRowChunk, row_last - rc + 1);
    __syncthreads();  // the previous chunk's rows are no longer read
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      double t[kMaxDim], wk[kMaxDim];
      uint64_t r = (uint64_t)(rc + i);
      for (int k = last - 1; k >= 0; --k) {
        uint64_t digit;
        if (small) {
          const uint32_t qq = fdiv((uint32_t)r, fdn);
          digit = (uint32_t)r - qq * fdn.d;
          r = qq;
        } else {
          const uint64_t qq = r / (uint64_t)n;
          digit = r - qq * (uint64_t)n;
          r = qq;
        }
        const double x = gl ? __dadd_rn(__dmul_rn(g.half[k], __ldg(gl_nodes + digit)), g.mid[k])
                            : linspace_node<double>(g.a[k], g.b[k], g.step[k], n, (int64_t)digit);
        t[k] = fam_term<FAM, double>(fam, k, x);
        wk[k] = g.wscale[k] * (gl ? __ldg(gl_w + digit) : (double)nc_int(rule, (int64_t)digit, n));
      }
      double sv = 0.0, wo = 1.0;
      for (int k = 0; k < last; ++k) {
        sv = (k == 0) ? t[k] : sv + t[k];
        wo *= wk[k];
      }
      const RowFactor rf = row_factor<FAM>(fam, sv);
      rt.p[i] = rf.r1;
      rt.q[i] = rf.r2;
      rt.ok[i] = rf.ok;
      rt.s[i] = sv;
      rt.w[i] = wo * wlast;
    }
    __syncthreads();
    const int64_t c0 = max(begin, rc * n), c1 = min(end, (rc + nr) * n);
    for (int64_t base = c0 + (int64_t)threadIdx.x * kTabP; base < c1; base += (int64_t)blockDim.x * kTabP) {
      const int cnt = (int)min((int64_t)kTabP, c1 - base);
      int ri, j;
      if (small) {
        const uint32_t qq = fdiv((uint32_t)base, fdn);
        ri = (int)((int64_t)qq - rc);
        j = (int)((uint32_t)base - qq * fdn.d);
      } else {
        const int64_t qq = base / n;
        ri = (int)(qq - rc);
        j = (int)(base - qq * n);
      }
      double seg = 0.0, ga = 0.0;
      for (int e = 0; e < cnt; ++e) {
        if (rt.ok[ri]) {
          seg = tab_accum<FAM>(seg, rt.p[ri], rt.q[ri], tab, j);
        } else {  // a row whose factor is not a normal number: the direct formula
          const double x = gl ? __dadd_rn(__dmul_rn(g.half[last], __ldg(gl_nodes + j)), g.mid[last])
                              : linspace_node<double>(g.a[last], g.b[last], g.step[last], n, j);
          const double v = fam_outer<FAM, double>(fam, rt.s[ri] + fam_term<FAM, double>(fam, last, x));
          seg = fma(tab.w[j], v, seg);
        }
        if (++j == n32) {
          ga = fma(seg, rt.w[ri], ga);
          seg = 0.0;
          j = 0;
          ++ri;
        }
      }
      if (j != 0) ga = fma(seg, rt.w[ri], ga);
      acc_add(acc, ga);
    }
  }
  return acc;
}

// ------------------------------------------------ adjoint of the families
// F(s) and F'(s) of the outer function, without the factor c.
template <int FAM, typename T>
__device__ __forceinline__ void fam_outer_d(const Family<T>& f, T s, T& F, T& Fp) {
  if (FAM == TQ_FN_EXP_SUM) {
    F = exp(s + f.b);
    Fp = F;
  } else if (FAM == TQ_FN_GAUSSIAN) {
    F = exp(-s);
    Fp = -F;
  } else if (FAM == TQ_FN_OSCILLATORY) {
    T sn, cs;
    sincos((T)(2.0 * CUDART_PI) * f.b + s, &sn, &cs);
    F = cs;
    Fp = -sn;
  } else {
    F = s;
    Fp = (T)1;
  }
}

// g_k'(x), dg_k/da_k, dg_k/du_k
template <int FAM, typename T>
__device__ __forceinline__ void fam_term_d(const Family<T>& f, int k, T x, T& gp, T& ga, T& gu) {
  if (FAM == TQ_FN_GAUSSIAN) {
    const T dd = x - f.u[k];
    gp = (T)2 * f.a[k] * dd;
    ga = dd * dd;
    gu = -(T)2 * f.a[k] * dd;
  } else if (FAM == TQ_FN_SUM_SIN) {
    const T cs = cos(f.a[k] * x);
    gp = f.a[k] * cs;
    ga = x * cs;
    gu = (T)0;
  } else {
    gp = f.a[k];
    ga = x;
    gu = (T)0;
  }
}

// Sum of v over the CTA (fixed tree); valid in warp 0, lane 0.  sh: 32
// doubles of shared memory.
__device__ __forceinline__ double block_sum_tree(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;
}

}  // namespace tq
