// Adjoint of the fused tensor-product rules: the integral and its gradient
// with respect to the domain bounds and the integrand parameters, in one
// pass over the grid (reverse mode of I = sum_i W_i f(x_i; theta)); for one
// integral (tq_grid_adjoint) and for a batch of many (tq_batch_grid_adjoint).
//
// The reference differentiates through torch autograd over the materialised
// [n^d, d] graph (integration_grid.py:74-88 requires_grad branch,
// utils.py:36-52 _linspace_with_grads, gaussian.py:81-84 / :159-162).  With
// nodes x_ik = a_k + t_ik L_k (L_k = b_k - a_k; t = unit node: linspace(0,1)
// for Newton-Cotes, (r+1)/2 for Gauss) and weights W_i proportional to
// prod_k L_k:
//   dI/db_k =  I/L_k + sum_i W_i df/dx_k t_ik
//   dI/da_k = -I/L_k + sum_i W_i df/dx_k (1 - t_ik)
//   dI/dtheta = sum_i W_i df/dtheta.
// For the separable families f = c F(s), s = sum_k g_k(x_k):
//   df/dx_k = c F'(s) g_k'(x_k), df/da_k = c F'(s) dg_k/da_k, ...
// Outer-dimension factors g_k', dg_k/da_k, t_k are constant along a grid
// row, so a row segment only accumulates sum W F, sum W F' and the
// last-dimension terms; the outer terms are folded in once per segment.
//
// fp64 grids of at most kAdjTab nodes per dimension take every node's F and
// F' from a per-row factor and a last-dimension table (the identities of the
// forward kernels' row tables: exp(s + t) = exp(s) exp(t), cos(p + t) =
// cos p cos t - sin p sin t, sin(p + t) = sin p cos t + cos p sin t), so the
// outer function is evaluated once per row instead of once per node; every
// node's value is still formed and weighted.

#include <type_traits>

#include "tq_grid_common.cuh"

namespace tq {

constexpr int kAdjTab = 256;  // last-dimension nodes the adjoint's table holds
constexpr int kAdjP = 32;     // consecutive nodes per thread and strip (a whole row at 32 nodes)
constexpr int kOutDims = 3;   // outer dimensions the adjoint's outer tables hold (dim <= 4)
constexpr int kOutTab = 64;   // nodes per dimension the outer tables hold

// The function entries carry the node's weight w, so a node's weighted value
// and derivative cost one or two fused multiply-adds.
struct AdjTab {
  double w[kAdjTab];   // unscaled 1-D weight
  double t[kAdjTab];   // unit node
  double T1[kAdjTab];  // w exp(+-t) | w cos t | w sin(a x)
  double T2[kAdjTab];  // w sin t (oscillatory)
  double gp[kAdjTab], ga[kAdjTab], gu[kAdjTab];
  double gpt[kAdjTab];  // gp t (Gaussian, sum of sines; gp is a constant otherwise)
  // the entries of the exponential and oscillatory node loops as
  // double-floats (that loop runs on the FP32 pipe)
  F2 T1f[kAdjTab], T2f[kAdjTab], tf[kAdjTab], gaf[kAdjTab], gpf[kAdjTab], gptf[kAdjTab];
  // outer dimensions (dim - 1 <= kOutDims, n <= kOutTab): each node's term,
  // weight factor, derivative terms and unit coordinate, computed once per
  // table and looked up by every row instead of recomputed (same values)
  double otv[kOutDims][kOutTab], ow[kOutDims][kOutTab], ogp[kOutDims][kOutTab];
  double oga[kOutDims][kOutTab], ogu[kOutDims][kOutTab], ot[kOutDims][kOutTab];
};

// An unnormalised double-float accumulator hi + lo of the node loop.
struct F2Acc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(F2 v) {
    const F2 t = two_sum(hi, v.hi);
    hi = t.hi;
    lo = __fadd_rn(lo, __fadd_rn(t.lo, v.lo));
  }
  // += a * b (TwoProduct through an FMA plus the cross terms)
  __device__ __forceinline__ void add_prod(F2 a, F2 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const F2 t = two_sum(hi, p);
    hi = t.hi;
    lo = __fadd_rn(lo, __fadd_rn(t.lo, e));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
// a*b + s*(c*d) for s = +-1, as a normalised double-float
template <int S>
__device__ __forceinline__ F2 f2_two_products(F2 a, F2 b, F2 c, F2 d) {
  const float p1 = __fmul_rn(a.hi, b.hi);
  float e1 = __fmaf_rn(a.hi, b.hi, -p1);
  e1 = __fmaf_rn(a.hi, b.lo, e1);
  e1 = __fmaf_rn(a.lo, b.hi, e1);
  const float p2 = __fmul_rn(c.hi, d.hi);
  float e2 = __fmaf_rn(c.hi, d.hi, -p2);
  e2 = __fmaf_rn(c.hi, d.lo, e2);
  e2 = __fmaf_rn(c.lo, d.hi, e2);
  const F2 t = two_sum(p1, S > 0 ? p2 : -p2);
  return two_sum(t.hi, __fadd_rn(t.lo, S > 0 ? __fadd_rn(e1, e2) : __fsub_rn(e1, e2)));
}

// Everything a thread needs to walk the nodes of one integral.
template <typename T, bool GL, int DM>
struct AdjCtx {
  const Geo<T>* g;
  const Family<T>* fam;
  const uint64_t* rstride;
  int dim, rule;
  int64_t n;
  const double* gln;
  const double* glw;
  AdjTab* tab;
  bool use_tab;
  bool f2;    // every table entry within the double-float node loop's range
  bool otab;  // the outer tables hold this integral's outer dimensions
};

template <int DM>
struct AdjAcc {
  double F, Fp, Sx[DM], St[DM], Pa[DM], Pu[DM];
  __device__ void zero() {
    F = Fp = 0.0;
#pragma unroll
    for (int k = 0; k < DM; ++k) Sx[k] = St[k] = Pa[k] = Pu[k] = 0.0;
  }
  // accumulator i of 2 + 4 * dim (F, F', then Sx, St, Pa, Pu by dimension)
  __device__ double at(int i, int dim) const {
    if (i == 0) return F;
    if (i == 1) return Fp;
    const int q = (i - 2) / dim, k = (i - 2) - q * dim;
    double v = 0.0;
#pragma unroll
    for (int kk = 0; kk < DM; ++kk)
      if (kk == k) v = q == 0 ? Sx[kk] : q == 1 ? St[kk] : q == 2 ? Pa[kk] : Pu[kk];
    return v;
  }
};

// Sums every accumulator i < 2 + 4*dim over the CTA and stores the sums at
// out[i * out_stride] (fixed trees: warp shuffles, then warp order).  sh:
// kBlock/32 rows of 2 + 4*DM doubles.  Contains a barrier; ends with one.
template <int DM>
__device__ void adj_block_store(const AdjAcc<DM>& acc, int dim, double (*sh)[2 + 4 * DM], double* out,
                                int64_t out_stride) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nacc = 2 + 4 * dim;
  for (int i = 0; i < nacc; ++i) {
    double v = acc.at(i, dim);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < nacc) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w][threadIdx.x];
    out[threadIdx.x * out_stride] = t;
  }
  __syncthreads();
}

// Row factors of the table path: F = p*T1 (exp families), p*T1 - q*T2
// (oscillatory), p + T1 (sum of sines).
struct AdjRow {
  double p, q;
  bool ok;
};
template <int FAM>
__device__ __forceinline__ AdjRow adj_row(const Family<double>& f, double s) {
  AdjRow r;
  r.q = 0.0;
  r.ok = true;
  if (FAM == TQ_FN_OSCILLATORY) {
    sincos(2.0 * CUDART_PI * f.b + s, &r.q, &r.p);
  } else if (FAM == TQ_FN_SUM_SIN) {
    r.p = s;
  } else {
    r.p = exp(FAM == TQ_FN_GAUSSIAN ? -s : s + f.b);
    r.ok = normal_factor(r.p);
  }
  return r;
}
// w F and w F' of node j from the row's factors and the weighted entries.
template <int FAM>
__device__ __forceinline__ void adj_wvalue(const AdjRow& r, const AdjTab& tb, int j, double& WF, double& WFp) {
  if (FAM == TQ_FN_OSCILLATORY) {
    WF = fma(r.p, tb.T1[j], -(r.q * tb.T2[j]));   // w cos(p + t)
    WFp = -fma(r.q, tb.T1[j], r.p * tb.T2[j]);    // -w sin(p + t)
  } else if (FAM == TQ_FN_SUM_SIN) {
    WF = fma(r.p, tb.w[j], tb.T1[j]);
    WFp = tb.w[j];
  } else {
    WF = r.p * tb.T1[j];
    WFp = FAM == TQ_FN_GAUSSIAN ? -WF : WF;
  }
}

// The double-float node loop takes factors that are zero or within
// [2^-30, 2^30]: products of three such factors, and sums of a strip of
// them, stay far inside the float range.
__device__ __forceinline__ bool f2_factor_ok(double v) {
  const double a = fabs(v);
  return v == 0.0 || (a >= 0x1p-30 && a <= 0x1p30);
}

// Builds the last-dimension table (all threads of the CTA; ends with a
// barrier); returns, in every thread, bit 0: every entry is usable, bit 1:
// every entry is within the double-float loop's range.
template <typename T, bool GL, int FAM, int DM>
__device__ int adj_build_tab(const AdjCtx<T, GL, DM>& c) {
  const int last = c.dim - 1, n32 = (int)c.n;
  const T ustep = (T)1 / (T)(c.n - 1);
  int bad = 0, f2bad = 0;
  for (int j = threadIdx.x; j < n32; j += blockDim.x) {
    const T x = node_at<T, GL>(*c.g, last, c.n, j, c.gln);
    const double w = GL ? __ldg(c.glw + j) : (double)nc_int(c.rule, j, c.n);
    c.tab->w[j] = w;
    c.tab->t[j] = GL ? (double)(T)((__ldg(c.gln + j) + 1.0) * 0.5)
                     : (double)linspace_node<T>((T)0, (T)1, ustep, c.n, j);
    T gp, ga, gu;
    fam_term_d<FAM, T>(*c.fam, last, x, gp, ga, gu);
    c.tab->gp[j] = (double)gp;
    c.tab->ga[j] = (double)ga;
    c.tab->gu[j] = (double)gu;
    c.tab->gpt[j] = (double)gp * c.tab->t[j];
    c.tab->tf[j] = f2_from_double(c.tab->t[j]);
    c.tab->gaf[j] = f2_from_double(c.tab->ga[j]);
    c.tab->gpf[j] = f2_from_double(c.tab->gp[j]);
    c.tab->gptf[j] = f2_from_double(c.tab->gpt[j]);
    const double tv = (double)fam_term<FAM, T>(*c.fam, last, x);
    if (FAM == TQ_FN_OSCILLATORY) {
      double sn, cs;
      sincos(tv, &sn, &cs);
      c.tab->T1[j] = w * cs;
      c.tab->T2[j] = w * sn;
    } else if (FAM == TQ_FN_SUM_SIN) {
      c.tab->T1[j] = w * tv;
      c.tab->T2[j] = 0.0;
    } else {
      const double e = exp(FAM == TQ_FN_GAUSSIAN ? -tv : tv);
      c.tab->T1[j] = w * e;
      c.tab->T2[j] = 0.0;
      bad |= !normal_factor(e) || !normal_factor(w * e);
    }
    c.tab->T1f[j] = f2_from_double(c.tab->T1[j]);
    c.tab->T2f[j] = f2_from_double(c.tab->T2[j]);
    f2bad |= !f2_factor_ok(c.tab->T1[j]) || !f2_factor_ok(c.tab->T2[j]) || !f2_factor_ok(c.tab->t[j]) ||
             !f2_factor_ok(c.tab->ga[j]) || !f2_factor_ok(c.tab->gp[j]) || !f2_factor_ok(c.tab->gpt[j]);
  }
  if (c.dim - 1 <= kOutDims && c.n <= kOutTab) {
    for (int e = threadIdx.x; e < (c.dim - 1) * n32; e += blockDim.x) {
      const int k = e / n32, j = e - k * n32;
      const T x = node_at<T, GL>(*c.g, k, c.n, j, c.gln);
      c.tab->otv[k][j] = (double)fam_term<FAM, T>(*c.fam, k, x);
      c.tab->ow[k][j] = c.g->wscale[k] * (GL ? __ldg(c.glw + j) : (double)nc_int(c.rule, j, c.n));
      T gp, ga, gu;
      fam_term_d<FAM, T>(*c.fam, k, x, gp, ga, gu);
      c.tab->ogp[k][j] = (double)gp;
      c.tab->oga[k][j] = (double)ga;
      c.tab->ogu[k][j] = (double)gu;
      c.tab->ot[k][j] = GL ? (double)(T)((__ldg(c.gln + j) + 1.0) * 0.5)
                           : (double)linspace_node<T>((T)0, (T)1, ustep, c.n, j);
    }
  }
  const int usable = !__syncthreads_or(bad);
  return usable | (__syncthreads_or(f2bad) ? 0 : 2);
}

// Adds the nodes [first, end) visited in strips of kAdjP starting at
// first, first + step, ... (flat indices, last dimension fastest).
template <typename T, bool GL, int FAM, int DM>
__device__ void adj_accumulate(const AdjCtx<T, GL, DM>& c, int64_t first, int64_t end, int64_t step,
                               AdjAcc<DM>& acc) {
  const Geo<T>& g = *c.g;
  const Family<T>& fam = *c.fam;
  const int dim = c.dim, last = dim - 1;
  const int64_t n = c.n;
  const int n32 = (int)n;
  const double wlast = g.wscale[last];
  const T ustep = (T)1 / (T)(n - 1);
  auto unit = [&](int64_t j) -> T {
    if (GL) return (T)((__ldg(c.gln + j) + 1.0) * 0.5);
    return linspace_node<T>((T)0, (T)1, ustep, n, j);
  };
  auto wunit = [&](int64_t j) -> double { return GL ? __ldg(c.glw + j) : (double)nc_int(c.rule, j, n); };
  for (int64_t base = first; base < end; base += step) {
    uint64_t row = (uint64_t)base / (uint64_t)n;
    int jl = (int)(base - (int64_t)row * n);
    int64_t left = min((int64_t)kAdjP, end - base);
    while (left > 0) {
      // outer-dimension state of this row: the separable sum and the weight
      // now, the per-dimension derivative factors after the segment (fewer
      // live registers across the node loop)
      T s_outer = T(0);
      double w_outer = 1.0;
      if (c.otab) {
        const AdjTab& tb = *c.tab;
#pragma unroll
        for (int k = 0; k < kOutDims; ++k) {
          if (k < dim - 1) {
            const int d = (int)((row / c.rstride[k]) % (uint64_t)n);
            const T tv = (T)tb.otv[k][d];
            s_outer = (k == 0) ? tv : s_outer + tv;
            w_outer *= tb.ow[k][d];
          }
        }
      } else {
#pragma unroll
        for (int k = 0; k < DM; ++k) {
          if (k < dim - 1) {
            const int64_t digit = (int64_t)((row / c.rstride[k]) % (uint64_t)n);
            const T x = node_at<T, GL>(g, k, n, digit, c.gln);
            const T tv = fam_term<FAM, T>(fam, k, x);
            s_outer = (k == 0) ? tv : s_outer + tv;
            w_outer *= g.wscale[k] * wunit(digit);
          }
        }
      }
      const int seg_end = (int)min((int64_t)n32, (int64_t)jl + left);
      double sF = 0.0, sFp = 0.0, sX = 0.0, sT = 0.0, sA = 0.0, sU = 0.0;
      bool tabbed = false;
      if constexpr (std::is_same<T, double>::value) {
        if (c.use_tab) {
          const AdjRow rf = adj_row<FAM>(fam, s_outer);
          if (rf.ok) {
            const AdjTab& tb = *c.tab;
            bool done = false;
            if constexpr (FAM != TQ_FN_SUM_SIN) {
              if (c.f2 && f2_factor_ok(rf.p) && f2_factor_ok(rf.q)) {
                // exponential and oscillatory families: the node terms and
                // their sums as double-floats on the FP32 pipe (about 2^-47
                // per operation); on GB300 the fp64 form of this loop (eight
                // FP64 instructions a node) was bound by the FP64 unit
                const F2 p = f2_from_double(rf.p), q = f2_from_double(rf.q);
                F2Acc aF, aFp, aX, aT, aA;
                for (int j = jl; j < seg_end; ++j) {
                  F2 WF, WFp;
                  if (FAM == TQ_FN_OSCILLATORY) {
                    WF = f2_two_products<-1>(p, tb.T1f[j], q, tb.T2f[j]);          // w cos(p + t)
                    const F2 sn = f2_two_products<1>(q, tb.T1f[j], p, tb.T2f[j]);  // w sin(p + t)
                    WFp = F2{-sn.hi, -sn.lo};
                  } else {
                    WF = f2_mul(p, tb.T1f[j]);
                    WFp = FAM == TQ_FN_GAUSSIAN ? F2{-WF.hi, -WF.lo} : WF;
                  }
                  aF.add(WF);
                  if (FAM == TQ_FN_OSCILLATORY) aFp.add(WFp);
                  if (FAM == TQ_FN_GAUSSIAN) {
                    aX.add_prod(WFp, tb.gpf[j]);
                    aT.add_prod(WFp, tb.gptf[j]);
                  } else {
                    aT.add_prod(WFp, tb.tf[j]);  // times the constant g' = a below
                  }
                  aA.add_prod(WFp, tb.gaf[j]);
                }
                sF = aF.value();
                sFp = FAM == TQ_FN_OSCILLATORY ? aFp.value() : (FAM == TQ_FN_GAUSSIAN ? -sF : sF);
                sX = aX.value();
                sT = aT.value();
                sA = aA.value();
                done = true;
              }
            }
            if (!done) {  // fp64: sums of sines, and factors outside the double-float range
              for (int j = jl; j < seg_end; ++j) {
                double WF, WFp;
                adj_wvalue<FAM>(rf, tb, j, WF, WFp);
                sF += WF;
                sFp += WFp;
                if (FAM == TQ_FN_GAUSSIAN || FAM == TQ_FN_SUM_SIN) {
                  sX = fma(WFp, tb.gp[j], sX);
                  sT = fma(WFp, tb.gpt[j], sT);
                } else {
                  sT = fma(WFp, tb.t[j], sT);  // times the constant g' = a below
                }
                sA = fma(WFp, tb.ga[j], sA);
              }
            }
            if (FAM == TQ_FN_GAUSSIAN) {
              sU = -sX;  // g'_u = -g'_x
            } else if (FAM != TQ_FN_SUM_SIN) {  // g = a x: g'_x = a, g'_u = 0
              const double al = (double)fam.a[last];
              sX = al * sFp;
              sT = al * sT;
            }
            tabbed = true;
          }
        }
      }
      if (!tabbed) {
        for (int j = jl; j < seg_end; ++j) {
          const T x = node_at<T, GL>(g, last, n, j, c.gln);
          T F, Fp, gp, ga, gu;
          fam_outer_d<FAM, T>(fam, s_outer + fam_term<FAM, T>(fam, last, x), F, Fp);
          fam_term_d<FAM, T>(fam, last, x, gp, ga, gu);
          const double W = wunit(j);
          const double wfp = W * (double)Fp;
          sF += W * (double)F;
          sFp += wfp;
          sX += wfp * (double)gp;
          sT += wfp * (double)gp * (double)unit(j);
          sA += wfp * (double)ga;
          sU += wfp * (double)gu;
        }
      }
      const double sc = w_outer * wlast;
      acc.F += sc * sF;
      acc.Fp += sc * sFp;
      const double fo = sc * sFp;
#pragma unroll
      for (int k = 0; k < DM; ++k) {
        if (k < dim - 1 && c.otab) {
          const int kk = k < kOutDims ? k : 0;  // k < dim - 1 <= kOutDims here
          const int d = (int)((row / c.rstride[kk]) % (uint64_t)n);
          const AdjTab& tb = *c.tab;
          const double gp_o = tb.ogp[kk][d];
          acc.Sx[k] += fo * gp_o;
          acc.St[k] += fo * gp_o * tb.ot[kk][d];
          acc.Pa[k] += fo * tb.oga[kk][d];
          acc.Pu[k] += fo * tb.ogu[kk][d];
        } else if (k < dim - 1) {
          const int64_t digit = (int64_t)((row / c.rstride[k]) % (uint64_t)n);
          const T x = node_at<T, GL>(g, k, n, digit, c.gln);
          T gp_o, ga_o, gu_o;
          fam_term_d<FAM, T>(fam, k, x, gp_o, ga_o, gu_o);
          const T t_o = unit(digit);
          acc.Sx[k] += fo * (double)gp_o;
          acc.St[k] += fo * (double)gp_o * (double)t_o;
          acc.Pa[k] += fo * (double)ga_o;
          acc.Pu[k] += fo * (double)gu_o;
        } else if (k == last) {
          acc.Sx[k] += sc * sX;
          acc.St[k] += sc * sT;
          acc.Pa[k] += sc * sA;
          acc.Pu[k] += sc * sU;
        }
      }
      left -= seg_end - jl;
      jl = 0;
      ++row;
    }
  }
}

// The integral and its gradients from the reduced accumulators tot[2+4*dim]
// (one thread).
template <typename D>
__device__ void adj_outputs(const double* tot, int family, double c, const D* dom, int dim,
                            double* out_value, double* out_gdom, double* out_gpar) {
  const double I = c * tot[0];
  *out_value = I;
  for (int k = 0; k < dim; ++k) {
    const double L = (double)dom[2 * k + 1] - (double)dom[2 * k];
    const double sx = c * tot[2 + k], st = c * tot[2 + dim + k];
    out_gdom[2 * k] = -I / L + (sx - st);
    out_gdom[2 * k + 1] = I / L + st;
    out_gpar[2 + k] = c * tot[2 + 2 * dim + k];
    out_gpar[2 + dim + k] = c * tot[2 + 3 * dim + k];
  }
  out_gpar[0] = tot[0];
  if (family == TQ_FN_EXP_SUM)
    out_gpar[1] = c * tot[0];
  else if (family == TQ_FN_OSCILLATORY)
    out_gpar[1] = 2.0 * CUDART_PI * c * tot[1];
  else
    out_gpar[1] = 0.0;
}

// ----------------------------------------------------------- one integral
struct GradArgs {
  int rule, dim, family;
  int64_t n, total;
  const void* domain;
  const double* gl_nodes;
  const double* gl_weights;
  const double* params;
  double* partials;  // [blocks][nacc]
  unsigned* ticket;
  double* out_value;
  double* out_gdom;  // [dim][2]
  double* out_gpar;  // [2 + 2*dim]
};

template <typename T, typename D, bool GL, int FAM, int DM>
__global__ void __launch_bounds__(kBlock) grid_adjoint_kernel(GradArgs args) {
  __shared__ Geo<T> g;
  __shared__ Family<T> fam;
  __shared__ uint64_t rstride[kMaxDim];
  __shared__ double sh[kBlock / 32][2 + 4 * DM];
  __shared__ AdjTab tab;
  if (threadIdx.x == 0) {
    geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
    load_family<T>(fam, args.family, args.dim, args.params);
    uint64_t st = 1;
    for (int k = args.dim - 2; k >= 0; --k) {
      rstride[k] = st;
      st *= (uint64_t)args.n;
    }
  }
  __syncthreads();
  AdjCtx<T, GL, DM> c{&g, &fam, rstride, args.dim, args.rule, args.n, args.gl_nodes, args.gl_weights, &tab,
                      false, false, false};
  if (std::is_same<T, double>::value && args.dim >= 2 && args.n <= kAdjTab)
  {
    const int tb = adj_build_tab<T, GL, FAM, DM>(c);
    c.use_tab = (tb & 1) != 0;
    c.f2 = (tb & 2) != 0;
    c.otab = c.use_tab && c.dim - 1 <= kOutDims && c.n <= kOutTab;
  }
  AdjAcc<DM> acc;
  acc.zero();
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  adj_accumulate<T, GL, FAM, DM>(c, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kAdjP, args.total,
                                 nthreads * kAdjP, acc);

  // per-CTA sums of the nacc = 2 + 4 * dim accumulators
  const int dim = args.dim, nacc = 2 + 4 * dim;
  adj_block_store<DM>(acc, dim, sh, args.partials + (int64_t)blockIdx.x * nacc, 1);
  if (last_block_arrives(args.ticket)) {
    // each warp reduces accumulators over the CTAs (strided, compensated,
    // fixed merge order)
    __shared__ double tot[2 + 4 * kMaxDim];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = warp; i < nacc; i += blockDim.x >> 5) {
      Acc a{0.0, 0.0};
      for (unsigned b = lane; b < gridDim.x; b += 32) acc_add(a, args.partials[(int64_t)b * nacc + i]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc_merge(a, acc_shfl_down(a, o));
      if (lane == 0) tot[i] = a.s + a.c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      adj_outputs<D>(tot, FAM, (double)fam.c, (const D*)args.domain, dim, args.out_value, args.out_gdom,
                     args.out_gpar);
      *args.ticket = 0u;
    }
  }
}

// ---------------------------------------------------------- many integrals
// Tiles of tile_pts consecutive nodes of one integral (the tq_batch_grid
// layout); each tile's 2 + 4*dim sums go to its row of partials, and a
// second kernel reduces every integral's rows in tile order.
struct BatchGradArgs {
  const tq_batch_desc* desc;
  const int64_t* tile_start;
  int64_t n_int, n_tiles, tile_pts;
  const double* params;
  const void* domains;
  const double* gl_nodes;
  const double* gl_weights;
  int family;
  int stride;        // partial sums per tile row: 2 + 4 * DM
  double* partials;  // [n_tiles][stride]
};

template <typename T, typename D, bool GL, int FAM, int DM>
__device__ void batch_adj_tile(const BatchGradArgs& a, const tq_batch_desc& d, int64_t tile, int64_t tile0,
                               const Geo<T>& g, const Family<T>& fam, const uint64_t* rstride, AdjTab* tab,
                               double (*sh)[2 + 4 * DM]) {
  AdjCtx<T, GL, DM> c{&g, &fam, rstride, d.dim, d.rule, d.n, a.gl_nodes + d.gl_off, a.gl_weights + d.gl_off,
                      tab, false, false, false};
  if (std::is_same<T, double>::value && d.dim >= 2 && d.n <= kAdjTab)
  {
    const int tb = adj_build_tab<T, GL, FAM, DM>(c);
    c.use_tab = (tb & 1) != 0;
    c.f2 = (tb & 2) != 0;
    c.otab = c.use_tab && c.dim - 1 <= kOutDims && c.n <= kOutTab;
  }
  const int64_t begin = (tile - tile0) * a.tile_pts;
  const int64_t end = min(d.total, begin + a.tile_pts);
  AdjAcc<DM> acc;
  acc.zero();
  adj_accumulate<T, GL, FAM, DM>(c, begin + (int64_t)threadIdx.x * kAdjP, end,
                                 (int64_t)blockDim.x * kAdjP, acc);
  adj_block_store<DM>(acc, d.dim, sh, a.partials + tile * a.stride, 1);
}

// Tile body of one (node type, rule kind) for the tile's family.
template <typename T, typename D, bool GL, int DM>
__device__ void batch_adj_dispatch(const BatchGradArgs& a, const tq_batch_desc& d, int64_t tile, int64_t tile0,
                                   const Geo<T>& g, const Family<T>& fam, const uint64_t* rstride, AdjTab* tab,
                                   double (*sh)[2 + 4 * DM]) {
  switch (fam.id) {
    case TQ_FN_EXP_SUM:
      batch_adj_tile<T, D, GL, TQ_FN_EXP_SUM, DM>(a, d, tile, tile0, g, fam, rstride, tab, sh);
      break;
    case TQ_FN_GAUSSIAN:
      batch_adj_tile<T, D, GL, TQ_FN_GAUSSIAN, DM>(a, d, tile, tile0, g, fam, rstride, tab, sh);
      break;
    case TQ_FN_OSCILLATORY:
      batch_adj_tile<T, D, GL, TQ_FN_OSCILLATORY, DM>(a, d, tile, tile0, g, fam, rstride, tab, sh);
      break;
    default:
      batch_adj_tile<T, D, GL, TQ_FN_SUM_SIN, DM>(a, d, tile, tile0, g, fam, rstride, tab, sh);
      break;
  }
}

// Gauss integrals and fp64 batches work in fp64 (their table rows as
// double-floats); fp32 Newton-Cotes integrals in fp32 (the node arithmetic
// of tq_grid_adjoint).  Up to four dimensions the kernel is held to 128
// registers, two CTAs per SM (a few hundred bytes of spills, 20 % faster
// than one CTA at 159 registers).
template <typename D, int DM>
__global__ void __launch_bounds__(kBlock, DM <= 4 ? 2 : 1) batch_adjoint_kernel(BatchGradArgs a) {
  __shared__ Geo<double> g64;
  __shared__ Family<double> fam64;
  __shared__ Geo<float> g32;
  __shared__ Family<float> fam32;
  __shared__ uint64_t rstride[kMaxDim];
  __shared__ double sh[kBlock / 32][2 + 4 * DM];
  __shared__ AdjTab tab;
  __shared__ tq_batch_desc d;
  __shared__ int64_t tile0;
  constexpr bool kF32 = std::is_same<D, float>::value;
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
      const int fid = a.family >= 0 ? a.family : d.family;
      const D* dom = (const D*)a.domains + d.dom_off;
      if (kF32 && d.rule != TQ_RULE_GAUSS) {
        geo_setup<float, D>(g32, d.rule, d.dim, d.n, dom);
        load_family<float>(fam32, fid, d.dim, a.params + d.par_off);
      } else {
        geo_setup<double, D>(g64, d.rule, d.dim, d.n, dom);
        load_family<double>(fam64, fid, d.dim, a.params + d.par_off);
      }
      uint64_t st = 1;
      for (int k = d.dim - 2; k >= 0; --k) {
        rstride[k] = st;
        st *= (uint64_t)d.n;
      }
    }
    __syncthreads();
    if (d.rule == TQ_RULE_GAUSS)
      batch_adj_dispatch<double, D, true, DM>(a, d, tile, tile0, g64, fam64, rstride, &tab, sh);
    else if (kF32)
      batch_adj_dispatch<float, D, false, DM>(a, d, tile, tile0, g32, fam32, rstride, &tab, sh);
    else
      batch_adj_dispatch<double, D, false, DM>(a, d, tile, tile0, g64, fam64, rstride, &tab, sh);
    __syncthreads();
  }
}

// One warp per integral: compensated sums of its tile rows in tile order,
// then the value and gradients.
template <typename D>
__global__ void batch_adjoint_finalize_kernel(BatchGradArgs a, double* out_value, double* out_gdom,
                                              double* out_gpar) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  __shared__ double tot[kBlock / 32][2 + 4 * 8];
  if (w >= a.n_int) return;
  const tq_batch_desc d = a.desc[w];
  const int nacc = 2 + 4 * d.dim;
  const int64_t t0 = a.tile_start[w], t1 = a.tile_start[w + 1];
  for (int i = 0; i < nacc; ++i) {
    Acc s{0.0, 0.0};
    for (int64_t t = t0 + lane; t < t1; t += 32) acc_add(s, a.partials[t * a.stride + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc_merge(s, acc_shfl_down(s, o));
    if (lane == 0) tot[wib][i] = s.s + s.c;
  }
  __syncwarp();
  if (lane == 0) {
    const int fid = a.family >= 0 ? a.family : d.family;
    adj_outputs<D>(tot[wib], fid, a.params[d.par_off], (const D*)a.domains + d.dom_off, d.dim, out_value + w,
                   out_gdom + d.dom_off, out_gpar + d.par_off);
  }
}

}  // namespace tq

using namespace tq;

static int64_t adj_blocks(int64_t total) {
  const int64_t need = (total + (int64_t)kBlock * kAdjP - 1) / ((int64_t)kBlock * kAdjP);
  const int64_t cap = (int64_t)sm_count() * 4;
  return need < 1 ? 1 : (need < cap ? need : cap);
}

static bool valid_nc(int rule, int64_t n) {
  if (rule < TQ_RULE_TRAPEZOID || rule > TQ_RULE_GAUSS || n < 2) return false;
  if (rule == TQ_RULE_SIMPSON && (n < 3 || !(n & 1))) return false;
  if (rule == TQ_RULE_BOOLE && (n < 5 || (n - 1) % 4)) return false;
  return true;
}

extern "C" size_t tq_grid_adjoint_workspace_size(int dim, int64_t total_points) {
  return 256 + (size_t)adj_blocks(total_points) * (2 + 4 * (size_t)(dim > 0 ? dim : 1)) * 8;
}

extern "C" int tq_grid_adjoint(int dtype, int rule, int dim, int64_t n_per_dim, const void* domain,
                               const double* gl_nodes, const double* gl_weights, int family,
                               const double* params, double* out_value, double* out_grad_domain,
                               double* out_grad_params, void* workspace, size_t workspace_bytes,
                               void* stream) {
  if (!valid_dtype(dtype)) return TQ_ERR_DTYPE;
  if (dim < 1 || dim > 8) return TQ_ERR_DIM;
  if (!valid_nc(rule, n_per_dim)) return TQ_ERR_RULE;
  if (!domain || !params || !out_value || !out_grad_domain || !out_grad_params || !workspace)
    return TQ_ERR_ARG;
  if (rule == TQ_RULE_GAUSS && (!gl_nodes || !gl_weights)) return TQ_ERR_ARG;
  int64_t total = 1;
  for (int k = 0; k < dim; ++k) {
    if (total > (int64_t(1) << 62) / n_per_dim) return TQ_ERR_TOO_LARGE;
    total *= n_per_dim;
  }
  if (workspace_bytes < tq_grid_adjoint_workspace_size(dim, total)) return TQ_ERR_WORKSPACE;
  GradArgs a;
  a.rule = rule;
  a.dim = dim;
  a.family = family;
  a.n = n_per_dim;
  a.total = total;
  a.domain = domain;
  a.gl_nodes = gl_nodes;
  a.gl_weights = gl_weights;
  a.params = params;
  a.ticket = (unsigned*)workspace;
  a.partials = (double*)((char*)workspace + 256);
  a.out_value = out_value;
  a.out_gdom = out_grad_domain;
  a.out_gpar = out_grad_params;
  const dim3 grid((unsigned)adj_blocks(total));
  cudaStream_t s = (cudaStream_t)stream;
#define TQ_ADJ(DMV)                                                                      \
  if (rule == TQ_RULE_GAUSS) {                                                           \
    if (dtype == TQ_F64)                                                                 \
      grid_adjoint_kernel<double, double, true, FAM, DMV><<<grid, kBlock, 0, s>>>(a);    \
    else                                                                                 \
      grid_adjoint_kernel<double, float, true, FAM, DMV><<<grid, kBlock, 0, s>>>(a);     \
  } else if (dtype == TQ_F64) {                                                          \
    grid_adjoint_kernel<double, double, false, FAM, DMV><<<grid, kBlock, 0, s>>>(a);     \
  } else {                                                                               \
    grid_adjoint_kernel<float, float, false, FAM, DMV><<<grid, kBlock, 0, s>>>(a);       \
  }
  TQ_DISPATCH_FAMILY(family, FAM, {
    if (dim <= 4) {
      TQ_ADJ(4)
    } else {
      TQ_ADJ(8)
    }
  });
#undef TQ_ADJ
  return launch_status();
}

extern "C" size_t tq_batch_grid_adjoint_workspace_size(int64_t n_tiles, int max_dim) {
  if (n_tiles < 1 || max_dim < 1 || max_dim > 8) return 0;
  const int dm = max_dim <= 4 ? 4 : 8;
  return (size_t)n_tiles * (2 + 4 * (size_t)dm) * sizeof(double);
}

extern "C" int tq_batch_grid_adjoint(int dtype, int64_t n_integrals, const void* descs,
                                     const int64_t* tile_start, int64_t n_tiles, int64_t tile_points,
                                     const double* params, const void* domains, const double* gl_nodes,
                                     const double* gl_weights, int family, int max_dim, double* out_value,
                                     double* out_grad_domain, double* out_grad_params, void* workspace,
                                     size_t workspace_bytes, void* stream) {
  if (!valid_dtype(dtype)) return TQ_ERR_DTYPE;
  if (max_dim < 1 || max_dim > 8) return TQ_ERR_DIM;
  if (family != TQ_FN_PER_DESC && (family < TQ_FN_EXP_SUM || family > TQ_FN_SUM_SIN)) return TQ_ERR_FAMILY;
  if (n_integrals < 1 || n_tiles < 1 || tile_points < 1 || !descs || !tile_start || !params || !domains ||
      !out_value || !out_grad_domain || !out_grad_params || !workspace)
    return TQ_ERR_ARG;
  const size_t need = tq_batch_grid_adjoint_workspace_size(n_tiles, max_dim);
  if (workspace_bytes < need) return TQ_ERR_WORKSPACE;
  BatchGradArgs a;
  a.desc = (const tq_batch_desc*)descs;
  a.tile_start = tile_start;
  a.n_int = n_integrals;
  a.n_tiles = n_tiles;
  a.tile_pts = tile_points;
  a.params = params;
  a.domains = domains;
  a.gl_nodes = gl_nodes ? gl_nodes : params;  // unused unless an integral is Gauss
  a.gl_weights = gl_weights ? gl_weights : params;
  a.family = family;
  a.stride = 2 + 4 * (max_dim <= 4 ? 4 : 8);
  a.partials = (double*)workspace;
  int64_t grid = (int64_t)sm_count() * 4;
  if (grid > n_tiles) grid = n_tiles;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned g = (unsigned)grid;
  if (dtype == TQ_F64) {
    if (max_dim <= 4) batch_adjoint_kernel<double, 4><<<g, kBlock, 0, s>>>(a);
    else batch_adjoint_kernel<double, 8><<<g, kBlock, 0, s>>>(a);
  } else {
    if (max_dim <= 4) batch_adjoint_kernel<float, 4><<<g, kBlock, 0, s>>>(a);
    else batch_adjoint_kernel<float, 8><<<g, kBlock, 0, s>>>(a);
  }
  int e = launch_status();
  if (e != TQ_OK) return e;
  const unsigned fb = (unsigned)((n_integrals * 32 + kBlock - 1) / kBlock);
  if (dtype == TQ_F64)
    batch_adjoint_finalize_kernel<double><<<fb, kBlock, 0, s>>>(a, out_value, out_grad_domain, out_grad_params);
  else
    batch_adjoint_finalize_kernel<float><<<fb, kBlock, 0, s>>>(a, out_value, out_grad_domain, out_grad_params);
  return launch_status();
}
