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

#include <type_traits>

#include "tq_grid_common.cuh"

namespace tq {

struct BatchDesc {
  int32_t rule, dim;
  int64_t n, total;
  int64_t par_off;  // into params (fp64, 2 + 2*dim values)
  int64_t dom_off;  // into domains (dtype, 2*dim values)
  int64_t gl_off;   // into gl_nodes / gl_weights (Gauss only)
  int32_t family;   // TQ_FN_* of this integral (used when the launch's family is TQ_FN_PER_DESC)
  int32_t pad;
};
static_assert(sizeof(BatchDesc) == sizeof(tq_batch_desc), "BatchDesc layout");

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

// Sum of one tile of the integral described by d (geometry g, family fam
// and rstride set up in shared memory by the caller); valid in thread 0.
template <typename T, int FAM, int P>
__device__ Acc grid_tile_sum(const BatchArgs& a, const BatchDesc& d, int64_t tile, int64_t tile0,
                             const Geo<T>& g, const Family<T>& fam, const uint64_t* rstride,
                             InnerTab* tab, RowTab* rt, FastDiv* fdn, const F2* wsf) {
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
  // fp64: last-dimension tables of this tile's integral (one
  // outer-function evaluation per row)
  bool use_tab = false;
  if constexpr (std::is_same<T, double>::value) {
    if (dim >= 2 && n <= kTabMax) use_tab = build_inner_tab<FAM>(*tab, g, fam, last, n32, gl, rule, gln, glw);
  }
  Acc acc{0.0, 0.0};
  RecurConst rc{1.0, 1.0, 0.0};
  if constexpr (std::is_same<T, double>::value) {
    if (use_tab) {
      if (threadIdx.x == 0) *fdn = make_fastdiv((uint32_t)n);
      __syncthreads();
      acc = tab_rows_sum<FAM>(g, fam, *tab, *rt, dim, rule, gl, n, *fdn, gln, glw, begin, end);
      return block_reduce<256>(acc);
    }
    // rows without a table (one dimension, or longer than a table): equally
    // spaced nodes by recurrence along the row
    if (!gl) rc = recur_const<FAM>(fam, last, st_l);
  }
  // node indices of an integral below 2^32: 32-bit divisions
  const bool small = d.total <= (int64_t)0xffffffffll;
  if constexpr (std::is_same<T, float>::value) {
    // fp32: the row weights and the running sums as double-floats on the
    // FP32 pipe (wsf: each dimension's weight scale); one conversion to
    // fp64 per thread and tile.  (fp64 arithmetic per row segment made this
    // path FP64-bound on GB300.)
    F2 facc{0.f, 0.f};
    // Gauss-Legendre: the last dimension's nodes and weights rounded to
    // fp32 once per tile (fp64 node mapping, as per node before)
    __shared__ float glx[kTabMax], glwf[kTabMax];
    const bool gl_tab = gl && n <= kTabMax;
    if (gl_tab) {
      for (int j = threadIdx.x; j < n32; j += blockDim.x) {
        glx[j] = (float)__dadd_rn(__dmul_rn(g.half[last], __ldg(gln + j)), g.mid[last]);
        glwf[j] = __double2float_rn(__ldg(glw + j));
      }
      __syncthreads();
    }
    for (int64_t base = begin + (int64_t)threadIdx.x * P; base < end; base += (int64_t)blockDim.x * P) {
      uint64_t row = small ? (uint64_t)((uint32_t)base / (uint32_t)n) : (uint64_t)base / (uint64_t)n;
      int jl = (int)(base - (int64_t)row * n);
      int64_t left = min((int64_t)P, end - base);
      while (left > 0) {
        float s_outer = 0.f;
        F2 w_outer{1.f, 0.f};
        for (int k = 0; k < dim - 1; ++k) {
          const int64_t digit = small ? (int64_t)(((uint32_t)row / (uint32_t)rstride[k]) % (uint32_t)n)
                                      : (int64_t)((row / rstride[k]) % (uint64_t)n);
          const float x = gl ? (float)__dadd_rn(__dmul_rn(g.half[k], __ldg(gln + digit)), g.mid[k])
                             : linspace_node<float>(g.a[k], g.b[k], g.step[k], n, digit);
          const float t = fam_term<FAM, float>(fam, k, x);
          s_outer = (k == 0) ? t : s_outer + t;
          w_outer = f2_mul(w_outer, wsf[k]);
          w_outer = gl ? f2_mul(w_outer, f2_from_double(__ldg(glw + digit)))
                       : f2_mul(w_outer, nc_coef_f(rule, (int)digit, n32));
        }
        const int seg_end = (int)min((int64_t)n32, (int64_t)jl + left);
        float sum = 0.f, comp = 0.f;
        // the node index as a float, stepped by one (exact below 2^24; one
        // conversion per segment instead of one per node)
        float fj = (float)jl;
        const float fn1 = (float)(n32 - 1);
        for (int j = jl; j < seg_end; ++j, fj += 1.f) {
          float x, wj;
          if (gl_tab) {
            x = glx[j];
            wj = glwf[j];
          } else if (gl) {
            x = (float)__dadd_rn(__dmul_rn(g.half[last], __ldg(gln + j)), g.mid[last]);
            wj = __double2float_rn(__ldg(glw + j));
          } else {
            x = (j < half) ? fmaf(st_l, fj, a_l) : fmaf(-st_l, fn1 - fj, b_l);
            wj = nc_coef_f(rule, j, n32);
          }
          const float f = fam_outer<FAM, float>(fam, s_outer + fam_term<FAM, float>(fam, last, x));
          // Kahan within the segment
          const float y = wj * f - comp;
          const float tt = sum + y;
          comp = (tt - sum) - y;
          sum = tt;
        }
        facc = f2_add(facc, f2_mul(f2_mul(two_sum(sum, -comp), w_outer), wsf[last]));
        left -= seg_end - jl;
        jl = 0;
        ++row;
      }
    }
    acc_add(acc, f2_value(facc));
    acc = block_reduce<256>(acc);
    if (gl_tab) __syncthreads();  // the tables are rewritten by the next tile
    return acc;
  }
  for (int64_t base = begin + (int64_t)threadIdx.x * P; base < end; base += (int64_t)blockDim.x * P) {
    uint64_t row = small ? (uint64_t)((uint32_t)base / (uint32_t)n) : (uint64_t)base / (uint64_t)n;
    int jl = (int)(base - (int64_t)row * n);
    int64_t left = min((int64_t)P, end - base);
    while (left > 0) {
      T s_outer = T(0);
      double w_outer = 1.0;
      for (int k = 0; k < dim - 1; ++k) {
        const int64_t digit = small ? (int64_t)(((uint32_t)row / (uint32_t)rstride[k]) % (uint32_t)n)
                                    : (int64_t)((row / rstride[k]) % (uint64_t)n);
        const T x = gl ? (T)__dadd_rn(__dmul_rn(g.half[k], __ldg(gln + digit)), g.mid[k])
                       : linspace_node<T>(g.a[k], g.b[k], g.step[k], n, digit);
        const T t = fam_term<FAM, T>(fam, k, x);
        s_outer = (k == 0) ? t : s_outer + t;
        w_outer *= g.wscale[k] * (gl ? __ldg(glw + digit) : (double)nc_int(rule, digit, n));
      }
      const int seg_end = (int)min((int64_t)n32, (int64_t)jl + left);
      T sum = T(0), comp = T(0);
      bool tabbed = false;
      if constexpr (std::is_same<T, double>::value) {
        if (!gl) {
          double v;
          const double x0 = linspace_node<double>(a_l, b_l, st_l, n, jl);
          const double x1 = linspace_node<double>(a_l, b_l, st_l, n, seg_end - 1);
          if (recur_seg_rule<FAM>(rule, fam, rc, last, s_outer, x0, x1, st_l, jl, seg_end, n32, &v)) {
            sum = v;
            tabbed = true;
          }
        }
        if (use_tab) {
          const RowFactor rf = row_factor<FAM>(fam, s_outer);
          if (rf.ok) {
            for (int j = jl; j < seg_end; ++j) {
              const double y = tab_accum<FAM>(0.0, rf.r1, rf.r2, *tab, j) - comp;
              const double tt = sum + y;
              comp = (tt - sum) - y;
              sum = tt;
            }
            tabbed = true;
          }
        }
      }
      for (int j = tabbed ? seg_end : jl; j < seg_end; ++j) {
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
  return block_reduce<256>(acc);
}

// Persistent launch over the flat tile list.  The family of a tile's
// integral is the launch's (a.family >= 0) or its descriptor's, so one
// launch can mix families; the switch is uniform across a CTA.
template <typename T, int P>
__global__ void __launch_bounds__(256) batch_grid_kernel(BatchArgs a) {
  __shared__ Geo<T> g;
  __shared__ Family<T> fam;
  __shared__ uint64_t rstride[kMaxDim];
  __shared__ BatchDesc d;
  __shared__ int64_t tile0;
  InnerTab* tab = nullptr;
  RowTab* rt = nullptr;
  __shared__ FastDiv fdn;
  __shared__ F2 wsf[kMaxDim];  // fp32: the dimensions' weight scales as double-floats
  if constexpr (std::is_same<T, double>::value) {
    __shared__ InnerTab tab_s;
    __shared__ RowTab rt_s;
    tab = &tab_s;
    rt = &rt_s;
  }
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
      load_family<T>(fam, a.family >= 0 ? a.family : d.family, d.dim, a.params + d.par_off);
      uint64_t st = 1;
      for (int k = d.dim - 2; k >= 0; --k) {
        rstride[k] = st;
        st *= (uint64_t)d.n;
      }
      if constexpr (std::is_same<T, float>::value)
        for (int k = 0; k < d.dim; ++k) wsf[k] = f2_from_double(g.wscale[k]);
    }
    __syncthreads();
    Acc acc{CUDART_NAN, 0.0};  // an unknown family (rejected on the host) gives NaN
    switch (fam.id) {
      case TQ_FN_EXP_SUM:
        acc = grid_tile_sum<T, TQ_FN_EXP_SUM, P>(a, d, tile, tile0, g, fam, rstride, tab, rt, &fdn, wsf);
        break;
      case TQ_FN_GAUSSIAN:
        acc = grid_tile_sum<T, TQ_FN_GAUSSIAN, P>(a, d, tile, tile0, g, fam, rstride, tab, rt, &fdn, wsf);
        break;
      case TQ_FN_OSCILLATORY:
        acc = grid_tile_sum<T, TQ_FN_OSCILLATORY, P>(a, d, tile, tile0, g, fam, rstride, tab, rt, &fdn, wsf);
        break;
      case TQ_FN_SUM_SIN:
        acc = grid_tile_sum<T, TQ_FN_SUM_SIN, P>(a, d, tile, tile0, g, fam, rstride, tab, rt, &fdn, wsf);
        break;
      default:
        break;
    }
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
  if (family != TQ_FN_PER_DESC && (family < TQ_FN_EXP_SUM || family > TQ_FN_SUM_SIN)) return TQ_ERR_FAMILY;
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
#define TQ_BATCH(T, PV) batch_grid_kernel<T, PV><<<(unsigned)grid, block, 0, s>>>(a)
  if (dtype == TQ_F64) {
    if (strip == 4) TQ_BATCH(double, 4);
    else TQ_BATCH(double, 16);
  } else {
    if (strip == 4) TQ_BATCH(float, 4);
    else TQ_BATCH(float, 16);
  }
#undef TQ_BATCH
  int e = launch_status();
  if (e != TQ_OK) return e;
  const unsigned fb = (unsigned)((n_integrals * 32 + 255) / 256);
  batch_finalize_kernel<<<fb, 256, 0, s>>>(tile_start, n_integrals, (const Acc*)workspace, out,
                                           out_dtype);
  return launch_status();
}

// ------------------------------------------------------ batched Monte Carlo
// One chunk of points for each of many Monte Carlo integrations: request r
// evaluates its points [first_r, first_r + count_r) of its own Philox stream
// (seed_r, stream_r; point p uses the elements p*dim .. p*dim+dim-1, the
// layout of tq_uniform) and adds sum f and sum f^2 to its running
// compensated accumulators acc[r][0..3].  Tiles of tile_pts points;
// per-tile partials are reduced in tile order, so a request's sums do not
// depend on the other requests of the launch.

namespace tq {

struct McDesc {
  int32_t dim, family;  // family: TQ_FN_* of this request (launch family TQ_FN_PER_DESC)
  int64_t first, count;  // point range of this chunk
  uint64_t seed, sid;
  int64_t par_off, dom_off;
};

struct BatchMcArgs {
  const McDesc* desc;
  const int64_t* tile_start;
  int64_t n_req, n_tiles, tile_pts;
  const double* params;
  const void* domains;
  int family;
  Acc* partials;  // [n_tiles][2]
};

// Sums f and f^2 over one tile of the chunk described by d; valid in thread 0.
template <typename T, int FAM>
__device__ void mc_tile_sums(const McDesc& d, int64_t begin, int64_t end, const Family<T>& fam,
                             const T* lo, const T* wid, Acc& s1, Acc& s2) {
  constexpr int PB = Uniform<T>::per_block;
  const int dim = d.dim;
  F2 f1{0.f, 0.f}, f2{0.f, 0.f};  // fp32 running sums of f and f^2
  for (int64_t q = begin + threadIdx.x; q < end; q += blockDim.x) {
    const uint64_t p = (uint64_t)(d.first + q);
    const uint64_t e0 = p * (uint64_t)dim;
    const uint64_t blk0 = e0 / PB;
    const int lane0 = (int)(e0 % PB);
    int cur = -1;
    uint4 r = make_uint4(0, 0, 0, 0);
    T s = T(0);
    for (int k = 0; k < dim; ++k) {
      const int le = lane0 + k, bi = le / PB;
      if (bi != cur) {
        r = philox_block(d.seed, d.sid, blk0 + (uint64_t)bi);
        cur = bi;
      }
      const T u = Uniform<T>::from(r, le - bi * PB);
      const T x = u * wid[k] + lo[k];
      const T g = fam_term<FAM, T>(fam, k, x);
      s = (k == 0) ? g : s + g;
    }
    if constexpr (std::is_same<T, float>::value) {
      // fp32: f and f^2 (exactly, as a TwoProduct) into double-floats on the
      // FP32 pipe; fp64 sums per sample made this path FP64-bound on GB300
      const float f = fam_outer<FAM, T>(fam, s);
      const float ff = __fmul_rn(f, f);
      f1 = f2_add(f1, f);
      f2 = f2_add(f2_add(f2, ff), __fmaf_rn(f, f, -ff));
    } else {
      const double f = (double)fam_outer<FAM, T>(fam, s);
      acc_add(s1, f);
      acc_add(s2, f * f);
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    acc_add(s1, f2_value(f1));
    acc_add(s2, f2_value(f2));
  }
  s1 = block_reduce<256>(s1);
  s2 = block_reduce<256>(s2);
}

template <typename T>
__global__ void __launch_bounds__(256) batch_mc_kernel(BatchMcArgs a) {
  __shared__ Family<T> fam;
  __shared__ T lo[kMaxDim], wid[kMaxDim];
  __shared__ McDesc d;
  __shared__ int64_t tile0;
  for (int64_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
    if (threadIdx.x == 0) {
      int64_t l = 0, h = a.n_req;
      while (h - l > 1) {
        const int64_t m = (l + h) >> 1;
        if (a.tile_start[m] <= tile) l = m;
        else h = m;
      }
      d = a.desc[l];
      tile0 = a.tile_start[l];
      load_family<T>(fam, a.family >= 0 ? a.family : d.family, d.dim, a.params + d.par_off);
      const T* dom = (const T*)a.domains + d.dom_off;
      for (int k = 0; k < d.dim; ++k) {
        lo[k] = dom[2 * k];
        wid[k] = dom[2 * k + 1] - dom[2 * k];
      }
    }
    __syncthreads();
    const int64_t begin = (tile - tile0) * a.tile_pts;
    const int64_t end = min(d.count, begin + a.tile_pts);
    Acc s1{0.0, 0.0}, s2{0.0, 0.0};
    switch (fam.id) {
      case TQ_FN_EXP_SUM:
        mc_tile_sums<T, TQ_FN_EXP_SUM>(d, begin, end, fam, lo, wid, s1, s2);
        break;
      case TQ_FN_GAUSSIAN:
        mc_tile_sums<T, TQ_FN_GAUSSIAN>(d, begin, end, fam, lo, wid, s1, s2);
        break;
      case TQ_FN_OSCILLATORY:
        mc_tile_sums<T, TQ_FN_OSCILLATORY>(d, begin, end, fam, lo, wid, s1, s2);
        break;
      case TQ_FN_SUM_SIN:
        mc_tile_sums<T, TQ_FN_SUM_SIN>(d, begin, end, fam, lo, wid, s1, s2);
        break;
      default:
        s1.s = CUDART_NAN;
        break;
    }
    if (threadIdx.x == 0) {
      a.partials[2 * tile] = s1;
      a.partials[2 * tile + 1] = s2;
    }
    __syncthreads();
  }
}

__global__ void batch_mc_finalize_kernel(const int64_t* tile_start, int64_t n_req, const Acc* partials,
                                         double* acc) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n_req) return;
  Acc s1{0.0, 0.0}, s2{0.0, 0.0};
  for (int64_t t = tile_start[w] + lane; t < tile_start[w + 1]; t += 32) {
    acc_merge(s1, partials[2 * t]);
    acc_merge(s2, partials[2 * t + 1]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    acc_merge(s1, acc_shfl_down(s1, o));
    acc_merge(s2, acc_shfl_down(s2, o));
  }
  if (lane == 0) {
    Acc r1{acc[4 * w], acc[4 * w + 1]}, r2{acc[4 * w + 2], acc[4 * w + 3]};
    acc_merge(r1, s1);
    acc_merge(r2, s2);
    acc[4 * w] = r1.s;
    acc[4 * w + 1] = r1.c;
    acc[4 * w + 2] = r2.s;
    acc[4 * w + 3] = r2.c;
  }
}

}  // namespace tq

extern "C" int tq_batch_mc(int dtype, int64_t n_requests, const void* descs,
                           const int64_t* tile_start, int64_t n_tiles, int64_t tile_points,
                           const double* params, const void* domains, int family, double* acc,
                           void* workspace, size_t workspace_bytes, void* stream) {
  using namespace tq;
  if (!valid_dtype(dtype)) return TQ_ERR_DTYPE;
  if (n_requests < 1 || n_tiles < 1 || tile_points < 1 || !descs || !tile_start || !params ||
      !domains || !acc || !workspace)
    return TQ_ERR_ARG;
  if (workspace_bytes < (size_t)n_tiles * 2 * sizeof(Acc)) return TQ_ERR_WORKSPACE;
  if (family != TQ_FN_PER_DESC && (family < TQ_FN_EXP_SUM || family > TQ_FN_SUM_SIN)) return TQ_ERR_FAMILY;
  BatchMcArgs a;
  a.desc = (const McDesc*)descs;
  a.tile_start = tile_start;
  a.n_req = n_requests;
  a.n_tiles = n_tiles;
  a.tile_pts = tile_points;
  a.params = params;
  a.domains = domains;
  a.family = family;
  a.partials = (Acc*)workspace;
  int64_t grid = (int64_t)sm_count() * 8;
  if (grid > n_tiles) grid = n_tiles;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TQ_F64)
    batch_mc_kernel<double><<<(unsigned)grid, 256, 0, s>>>(a);
  else
    batch_mc_kernel<float><<<(unsigned)grid, 256, 0, s>>>(a);
  int e = launch_status();
  if (e != TQ_OK) return e;
  batch_mc_finalize_kernel<<<(unsigned)((n_requests * 32 + 255) / 256), 256, 0, s>>>(
      tile_start, n_requests, (const Acc*)workspace, acc);
  return launch_status();
}
