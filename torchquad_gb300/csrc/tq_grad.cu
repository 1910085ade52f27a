// Adjoint of the fused tensor-product rules: the integral and its gradient
// with respect to the domain bounds and the integrand parameters, in one
// pass over the grid (reverse mode of I = sum_i W_i f(x_i; theta)).
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

#include "tq_grid_common.cuh"

namespace tq {

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

template <typename T, typename D, bool GL, int FAM, int DM>
__global__ void __launch_bounds__(kBlock) grid_adjoint_kernel(GradArgs args) {
  __shared__ Geo<T> g;
  __shared__ Family<T> fam;
  __shared__ uint64_t rstride[kMaxDim];
  __shared__ double sh[kBlock / 32];
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
  const int dim = args.dim, last = dim - 1, rule = args.rule;
  const int64_t n = args.n, total = args.total;
  const int n32 = (int)n;
  const double wlast = g.wscale[last];
  const T ustep = (T)1 / (T)(n - 1);

  // unit node t in [0,1] of index j in a dimension (see header comment)
  auto unit = [&](int j) -> T {
    if (GL) return (T)((__ldg(args.gl_nodes + j) + 1.0) * 0.5);
    return linspace_node<T>((T)0, (T)1, ustep, n, j);
  };
  auto node = [&](int k, int64_t j) -> T { return node_at<T, GL>(g, k, n, j, args.gl_nodes); };
  auto wunit = [&](int64_t j) -> double {
    return GL ? __ldg(args.gl_weights + j) : (double)nc_int(rule, j, n);
  };

  double accF = 0.0, accFp = 0.0;
  double Sx[DM], St[DM], Pa[DM], Pu[DM];
#pragma unroll
  for (int k = 0; k < DM; ++k) Sx[k] = St[k] = Pa[k] = Pu[k] = 0.0;

  constexpr int P = 16;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * P; base < total;
       base += nthreads * P) {
    uint64_t row = (uint64_t)base / (uint64_t)n;
    int jl = (int)(base - (int64_t)row * n);
    int64_t left = min((int64_t)P, total - base);
    while (left > 0) {
      // outer-dimension state of this row
      T s_outer = T(0);
      double w_outer = 1.0;
      T gp_o[DM], ga_o[DM], gu_o[DM], t_o[DM];
#pragma unroll
      for (int k = 0; k < DM; ++k) gp_o[k] = ga_o[k] = gu_o[k] = t_o[k] = T(0);
#pragma unroll
      for (int k = 0; k < DM; ++k) {
        if (k < dim - 1) {
          const int64_t digit = (int64_t)((row / rstride[k]) % (uint64_t)n);
          const T x = node(k, digit);
          const T tv = fam_term<FAM, T>(fam, k, x);
          s_outer = (k == 0) ? tv : s_outer + tv;
          w_outer *= g.wscale[k] * wunit(digit);
          fam_term_d<FAM, T>(fam, k, x, gp_o[k], ga_o[k], gu_o[k]);
          t_o[k] = unit((int)digit);
        }
      }
      const int seg_end = (int)min((int64_t)n32, (int64_t)jl + left);
      double sF = 0.0, sFp = 0.0, sX = 0.0, sT = 0.0, sA = 0.0, sU = 0.0;
      for (int j = jl; j < seg_end; ++j) {
        const T x = node(last, j);
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
      const double sc = w_outer * wlast;
      accF += sc * sF;
      accFp += sc * sFp;
      const double fo = sc * sFp;
#pragma unroll
      for (int k = 0; k < DM; ++k) {
        if (k < dim - 1) {
          Sx[k] += fo * (double)gp_o[k];
          St[k] += fo * (double)gp_o[k] * (double)t_o[k];
          Pa[k] += fo * (double)ga_o[k];
          Pu[k] += fo * (double)gu_o[k];
        } else if (k == last) {
          Sx[k] += sc * sX;
          St[k] += sc * sT;
          Pa[k] += sc * sA;
          Pu[k] += sc * sU;
        }
      }
      left -= seg_end - jl;
      jl = 0;
      ++row;
    }
  }

  // per-CTA sums, one accumulator at a time: nacc = 2 + 4 * dim
  const int nacc = 2 + 4 * dim;
  auto acc_at = [&](int i) -> double {
    if (i == 0) return accF;
    if (i == 1) return accFp;
    const int q = (i - 2) / dim, k = (i - 2) - q * dim;
    double v = 0.0;
#pragma unroll
    for (int kk = 0; kk < DM; ++kk)
      if (kk == k) v = q == 0 ? Sx[kk] : q == 1 ? St[kk] : q == 2 ? Pa[kk] : Pu[kk];
    return v;
  };
  for (int i = 0; i < nacc; ++i) {
    const double t = block_sum_tree(acc_at(i), sh);
    if (threadIdx.x == 0) args.partials[(int64_t)blockIdx.x * nacc + i] = t;
  }
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
      const double c = (double)fam.c;
      const double I = c * tot[0];
      *args.out_value = I;
      const D* dom = (const D*)args.domain;
      for (int k = 0; k < dim; ++k) {
        const double L = (double)dom[2 * k + 1] - (double)dom[2 * k];
        const double sx = c * tot[2 + k], st = c * tot[2 + dim + k];
        args.out_gdom[2 * k] = -I / L + (sx - st);
        args.out_gdom[2 * k + 1] = I / L + st;
        args.out_gpar[2 + k] = c * tot[2 + 2 * dim + k];
        args.out_gpar[2 + dim + k] = c * tot[2 + 3 * dim + k];
      }
      args.out_gpar[0] = tot[0];
      if (FAM == TQ_FN_EXP_SUM)
        args.out_gpar[1] = c * tot[0];
      else if (FAM == TQ_FN_OSCILLATORY)
        args.out_gpar[1] = 2.0 * CUDART_PI * c * tot[1];
      else
        args.out_gpar[1] = 0.0;
      *args.ticket = 0u;
    }
  }
}

}  // namespace tq

using namespace tq;

static int64_t adj_blocks(int64_t total) {
  const int64_t need = (total + (int64_t)kBlock * 16 - 1) / ((int64_t)kBlock * 16);
  const int64_t cap = (int64_t)sm_count() * 4;
  return need < 1 ? 1 : (need < cap ? need : cap);
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
  if (rule < TQ_RULE_TRAPEZOID || rule > TQ_RULE_GAUSS) return TQ_ERR_RULE;
  if ((rule == TQ_RULE_SIMPSON && (n_per_dim < 3 || !(n_per_dim & 1))) ||
      (rule == TQ_RULE_BOOLE && (n_per_dim < 5 || (n_per_dim - 1) % 4)) || n_per_dim < 2)
    return TQ_ERR_RULE;
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
