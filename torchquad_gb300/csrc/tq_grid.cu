// Tensor-product quadrature on GB300: fused node generation + integrand +
// weighted sum for built-in integrands, and the node / weight / weighted-sum
// kernels of the materialised path used for arbitrary torch integrands.
//
// The reference builds the full [n^d, d] point tensor (integration_grid.py:
// 95-99), evaluates the integrand on it, transposes the values
// (grid_integrator.py:80) and collapses one dimension at a time
// (trapezoid.py:27-37, simpson.py:29-46, boole.py:29-48, gaussian.py:131-144).
// Here a thread walks a strip of consecutive flat node indices (last
// dimension fastest, the reference's meshgrid "ij" order), keeps the
// outer-dimension coordinates and weight product in registers, and sums
// w_i * f(x_i) directly; the per-dimension collapse becomes the product of
// 1-D weights, which is the same quadrature.

#include <type_traits>

#include "tq_grid_common.cuh"

namespace tq {

// ------------------------------------------------------------------ fused
struct FusedArgs {
  int rule, dim, family;
  int64_t n, total;
  const void* domain;
  const double* gl_nodes;
  const double* gl_weights;
  const double* params;
  Acc* partials;
  unsigned* ticket;
  void* out;
  int out_dtype;
  double* out64;
};

__device__ __forceinline__ void write_result(void* out, int out_dtype, double* out64,
                                             double v) {
  if (out) {
    if (out_dtype == TQ_F64)
      *(double*)out = v;
    else
      *(float*)out = (float)v;
  }
  if (out64) *out64 = v;
}

// Compensated sum of one row segment in the working type: Kahan's original
// four-operation update for fp32, plain accumulation for fp64 (a segment is
// at most n terms of one row).
template <typename T>
struct SegSum;
template <>
struct SegSum<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <>
struct SegSum<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};

// Outer-dimension state of a grid row (flat node index / n): the partial
// separable sum g_0 + ... + g_{d-2} in dimension order and the product of
// the outer 1-D weights.  rstride[k] = n^(dim-2-k).
template <typename T, int RULE, int FAM>
__device__ __forceinline__ void outer_state(const Geo<T>& g, const Family<T>& fam,
                                            const uint64_t* rstride, int dim, int64_t n,
                                            uint64_t row, const double* gl_nodes,
                                            const double* gl_w, bool small, T& s_out,
                                            double& w_out) {
  constexpr bool GL = RULE == TQ_RULE_GAUSS;
  T s = T(0);
  double w = 1.0;
#pragma unroll 1
  for (int k = 0; k < dim - 1; ++k) {
    uint64_t digit;
    if (small) {
      const uint32_t q = (uint32_t)row / (uint32_t)rstride[k];
      digit = q % (uint32_t)n;
    } else {
      digit = (row / rstride[k]) % (uint64_t)n;
    }
    const T x = node_at<T, GL>(g, k, n, (int64_t)digit, gl_nodes);
    const T t = fam_term<FAM, T>(fam, k, x);
    s = (k == 0) ? t : s + t;
    w *= g.wscale[k] *
         (GL ? __ldg(gl_w + digit) : (double)nc_int_t<RULE>((int)digit, (int)n));
  }
  s_out = s;
  w_out = w;
}

template <typename T, typename D, int RULE, int FAM, int P>
__global__ void __launch_bounds__(kBlock, 2) grid_fused_kernel(FusedArgs args) {
  constexpr bool GL = RULE == TQ_RULE_GAUSS;
  __shared__ Geo<T> g;
  __shared__ Family<T> fam;
  __shared__ uint64_t rstride[kMaxDim];
  if (threadIdx.x == 0) {
    geo_setup<T, D>(g, RULE, args.dim, args.n, (const D*)args.domain);
    load_family<T>(fam, args.family, args.dim, args.params);
    uint64_t st = 1;
    for (int k = args.dim - 2; k >= 0; --k) {
      rstride[k] = st;
      st *= (uint64_t)args.n;
    }
  }
  __syncthreads();
  const int dim = args.dim, last = dim - 1;
  const int64_t n = args.n, total = args.total;
  const int n32 = (int)n;  // n <= total < 2^62 but a row index fits int for n < 2^31
  const bool small = total < (int64_t(1) << 32);
  const double* gl_nodes = args.gl_nodes;
  const double* gl_w = args.gl_weights;
  const double wlast = g.wscale[last];
  const T a_l = g.a[last], b_l = g.b[last], st_l = g.step[last];
  const int half = n32 / 2;
  // fp64: last-dimension tables (one outer-function evaluation per row)
  bool use_tab = false;
  InnerTab* tab = nullptr;
  if constexpr (std::is_same<T, double>::value) {
    __shared__ InnerTab tab_s;
    tab = &tab_s;
    if (dim >= 2 && n <= kTabMax)
      use_tab = build_inner_tab<FAM>(tab_s, g, fam, last, n32, GL, RULE, gl_nodes, gl_w);
  }

  Acc acc{0.0, 0.0};
  bool rows_done = false;
  if constexpr (std::is_same<T, double>::value) {
    if (use_tab) {
      // a contiguous node range per CTA, rows in groups of 32 per warp
      __shared__ FastDiv fdn;
      __shared__ RowTab rt;
      if (threadIdx.x == 0) fdn = make_fastdiv((uint32_t)n);
      __syncthreads();
      const int64_t b0 = total * (int64_t)blockIdx.x / gridDim.x, b1 = total * ((int64_t)blockIdx.x + 1) / gridDim.x;
      if (b1 > b0) acc = tab_rows_sum<FAM>(g, fam, *tab, rt, dim, args.rule, GL, n, fdn, gl_nodes, gl_w, b0, b1);
      rows_done = true;
    }
  }
  RecurConst rc{1.0, 1.0, 0.0};
  if constexpr (std::is_same<T, double>::value) {
    if (!rows_done && !use_tab && !GL) rc = recur_const<FAM>(fam, last, st_l);
  }
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * P; base < total && !rows_done;
       base += nthreads * P) {
    uint64_t row;
    int jl;
    if (small) {
      const uint32_t q = (uint32_t)base / (uint32_t)n;
      row = q;
      jl = (int)((uint32_t)base - q * (uint32_t)n);
    } else {
      row = (uint64_t)base / (uint64_t)n;
      jl = (int)(base - (int64_t)row * n);
    }
    int64_t left = min((int64_t)P, total - base);
    while (left > 0) {
      T s_outer;
      double w_outer;
      outer_state<T, RULE, FAM>(g, fam, rstride, dim, n, row, gl_nodes, gl_w, small, s_outer,
                                w_outer);
      const int seg_end = (int)min((int64_t)n32, (int64_t)jl + left);
      SegSum<T> seg;
      bool tabbed = false;
      if constexpr (std::is_same<T, double>::value) {
        if (use_tab) {
          const RowFactor rf = row_factor<FAM>(fam, s_outer);
          if (rf.ok) {
            for (int j = jl; j < seg_end; ++j) seg.add(tab_accum<FAM>(0.0, rf.r1, rf.r2, *tab, j));
            tabbed = true;
          }
        } else if (!GL) {
          // rows without a table (one dimension, or longer than a table):
          // equally spaced nodes by recurrence along the row
          double v;
          const double x0 = linspace_node<double>(a_l, b_l, st_l, n, jl);
          const double x1 = linspace_node<double>(a_l, b_l, st_l, n, seg_end - 1);
          if (recur_seg<FAM, RULE>(fam, rc, last, s_outer, x0, x1, st_l, jl, seg_end, n32, &v)) {
            seg.add(v);
            tabbed = true;
          }
        }
      }
      if (!tabbed) {
        for (int j = jl; j < seg_end; ++j) {
          T x;
          if (GL)
            x = (T)__dadd_rn(__dmul_rn(g.half[last], __ldg(gl_nodes + j)), g.mid[last]);
          else
            x = (j < half) ? fma(st_l, (T)j, a_l) : fma(-st_l, (T)(n32 - 1 - j), b_l);
          const T f = fam_outer<FAM, T>(fam, s_outer + fam_term<FAM, T>(fam, last, x));
          const T wj = GL ? (T)__ldg(gl_w + j) : (T)nc_int_t<RULE>(j, n32);
          seg.add(wj * f);
        }
      }
      acc_add(acc, seg.value() * (w_outer * wlast));
      left -= seg_end - jl;
      jl = 0;
      ++row;
    }
  }

  acc = block_reduce<kBlock>(acc);
  if (threadIdx.x == 0) args.partials[blockIdx.x] = acc;
  if (last_block_arrives(args.ticket)) {
    Acc t{0.0, 0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) acc_merge(t, args.partials[i]);
    t = block_reduce<kBlock>(t);
    if (threadIdx.x == 0) {
      write_result(args.out, args.out_dtype, args.out64, t.s + t.c);
      *args.ticket = 0u;
    }
  }
}

// ------------------------------------------------------ materialised path
struct PointsArgs {
  int rule, dim;
  int64_t n, start, count;
  const void* domain;
  const double* gl_nodes;
  void* points;
};

// One thread per output element (point p, dimension k): coalesced stores of
// the [count, dim] row-major point tensor.
template <typename T, typename D, bool GL>
__global__ void __launch_bounds__(kBlock) grid_points_kernel(PointsArgs args) {
  __shared__ Geo<T> g;
  __shared__ uint64_t stride[kMaxDim];
  if (threadIdx.x == 0) {
    geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
    uint64_t s = 1;
    for (int k = args.dim - 1; k >= 0; --k) {
      stride[k] = s;
      s *= (uint64_t)args.n;
    }
  }
  __syncthreads();
  const int dim = args.dim;
  const uint64_t n = (uint64_t)args.n;
  const uint64_t numel = (uint64_t)args.count * dim;
  T* out = (T*)args.points;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < numel;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t p = e / (uint64_t)dim;
    const int k = (int)(e - p * dim);
    const uint64_t digit = ((args.start + p) / stride[k]) % n;
    out[e] = node_at<T, GL>(g, k, (int64_t)n, (int64_t)digit, args.gl_nodes);
  }
}

// Tiled variant (HBM-write bound): a CTA builds a tile of consecutive
// points in shared memory (one thread per point; digits by multiply-high
// division by n; node values from a per-CTA table of every dimension's
// nodes), then one thread hands the tile to the bulk-copy engine
// (cp.async.bulk shared -> global), so the stores are full-line writes
// issued without per-thread store instructions.  Two tile buffers alternate;
// a buffer is rewritten only after its previous copy has been read out
// (cp.async.bulk.wait_group.read 1).  Needs a 16-byte aligned output.
constexpr int kPtsTileBytes = 24 * 1024;  // per buffer (two buffers per CTA)
constexpr int kPtsTab = 2048;             // node-table entries (dim * n) a CTA keeps

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

template <typename T, typename D, bool GL>
__global__ void __launch_bounds__(kBlock) grid_points_tiled_kernel(PointsArgs args, int tile_pts,
                                                                   int64_t n_tiles) {
  extern __shared__ __align__(128) unsigned char pts_smem[];
  __shared__ Geo<T> g;
  __shared__ FastDiv fd_n;
  __shared__ T nodes[kPtsTab];  // nodes[k * n + j], when dim * n fits
  if (threadIdx.x == 0) {
    geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
    fd_n = make_fastdiv((uint32_t)args.n);
  }
  __syncthreads();
  const int dim = args.dim;
  const uint64_t n = (uint64_t)args.n;
  const int n32 = (int)args.n;
  // the nodes of every dimension once per CTA (no per-point node arithmetic)
  const bool tab = (int64_t)dim * args.n <= kPtsTab;
  if (tab)
    for (int e = threadIdx.x; e < dim * n32; e += blockDim.x)
      nodes[e] = node_at<T, GL>(g, e / n32, (int64_t)n, (int64_t)(e % n32), args.gl_nodes);
  // point indices below 2^32 (all but huge grids): 32-bit digits
  const bool small = (uint64_t)(args.start + args.count) <= 0xffffffffull;
  int buf = 0;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    T* sm = (T*)(pts_smem + (size_t)buf * kPtsTileBytes);
    const int64_t p0 = tile * (int64_t)tile_pts;  // local point index
    const int np = (int)min((int64_t)tile_pts, args.count - p0);
    if (threadIdx.x == 0) {
      // the copy that last read this buffer (two tiles ago) must be done
      asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
    }
    __syncthreads();
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
      const uint64_t idx = (uint64_t)(args.start + p0 + p);
      T* row = sm + (size_t)p * dim;
      if (small && tab) {
        uint32_t r = (uint32_t)idx;
        for (int k = dim - 1; k >= 0; --k) {
          const uint32_t q = fdiv(r, fd_n);
          row[k] = nodes[k * n32 + (int)(r - q * fd_n.d)];
          r = q;
        }
      } else {
        uint64_t r = idx;
        for (int k = dim - 1; k >= 0; --k) {
          const uint64_t q = r / n;
          row[k] = node_at<T, GL>(g, k, (int64_t)n, (int64_t)(r - q * n), args.gl_nodes);
          r = q;
        }
      }
    }
    // generic-proxy writes of the tile -> visible to the bulk copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    const size_t bytes = (size_t)np * dim * sizeof(T);
    const size_t bulk = bytes & ~(size_t)15;
    unsigned char* dst = (unsigned char*)args.points + (size_t)p0 * dim * sizeof(T);
    if (threadIdx.x == 0 && bulk > 0) {
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                   "r"(smem_u32(sm)), "r"((uint32_t)bulk)
                   : "memory");
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    }
    // a tail of 4, 8 or 12 bytes (only in the last tile) by plain stores
    for (size_t b = bulk + threadIdx.x * sizeof(T); b < bytes; b += blockDim.x * sizeof(T))
      *(T*)(dst + b) = *(const T*)((const unsigned char*)sm + b);
    buf ^= 1;
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

struct WeightsArgs {
  int rule, dim;
  int64_t n, start, count;
  const void* domain;
  const double* gl_weights;
  double* weights;
};

template <typename T, typename D, bool GL>
__global__ void __launch_bounds__(kBlock) grid_weights_kernel(WeightsArgs args) {
  __shared__ Geo<T> g;
  if (threadIdx.x == 0) geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
  __syncthreads();
  const int dim = args.dim;
  const uint64_t n = (uint64_t)args.n;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < (uint64_t)args.count;
       p += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t r = args.start + p;
    double w = 1.0;
    for (int k = dim - 1; k >= 0; --k) {
      const uint64_t q = r / n, digit = r - q * n;
      r = q;
      w *= g.wscale[k] * wunit_at<GL>(args.rule, (int64_t)n, (int64_t)digit, args.gl_weights);
    }
    args.weights[p] = w;
  }
}

// Weighted sum of materialised integrand values.  A thread walks a strip of
// consecutive nodes (weights by the same odometer as the fused kernel) and
// accumulates up to kVals integrand components; gridDim.y covers the
// components in groups of kVals.  Partials are reduced in fixed order by the
// last CTA and added to the running compensated sums acc[].
constexpr int kVals = 4;
struct WsumArgs {
  int rule, dim;
  int64_t n, start, count, n_values;
  const void* domain;
  const double* gl_weights;
  const void* f;
  double* acc;
  Acc* partials;  // [gridDim.x * gridDim.y][kVals]
  unsigned* ticket;
};

template <typename T, typename D, bool GL, typename F, int P>
__global__ void __launch_bounds__(kBlock) weighted_sum_kernel(WsumArgs args) {
  __shared__ Geo<T> g;
  if (threadIdx.x == 0) geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
  __syncthreads();
  const int dim = args.dim, rule = args.rule;
  const uint64_t n = (uint64_t)args.n;
  const int64_t S = args.n_values;
  const int64_t s0 = (int64_t)blockIdx.y * kVals;
  const int nv = (int)min((int64_t)kVals, S - s0);
  const F* __restrict__ f = (const F*)args.f;
  Acc acc[kVals];
#pragma unroll
  for (int v = 0; v < kVals; ++v) acc[v] = Acc{0.0, 0.0};

  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * P; base < args.count;
       base += nthreads * P) {
    const int64_t end = min(base + P, args.count);
    for (int64_t p = base; p < end; ++p) {
      double w = 1.0;
      if (rule != TQ_RULE_MC) {
        uint64_t r = (uint64_t)(args.start + p);
        for (int k = dim - 1; k >= 0; --k) {
          const uint64_t q = r / n, digit = r - q * n;
          r = q;
          w *= g.wscale[k] * wunit_at<GL>(rule, (int64_t)n, (int64_t)digit, args.gl_weights);
        }
      }
      const F* row = f + p * S + s0;
#pragma unroll
      for (int v = 0; v < kVals; ++v)
        if (v < nv) acc_add(acc[v], w * (double)row[v]);
    }
  }
  const int slot = blockIdx.y * gridDim.x + blockIdx.x;
#pragma unroll
  for (int v = 0; v < kVals; ++v) {
    Acc r = block_reduce<kBlock>(acc[v]);
    if (threadIdx.x == 0) args.partials[(int64_t)slot * kVals + v] = r;
  }
  if (last_block_arrives(args.ticket)) {
    // one component at a time, partials in index order
    for (int64_t s = 0; s < S; ++s) {
      const int64_t by = s / kVals;
      const int v = (int)(s - by * kVals);
      Acc t{0.0, 0.0};
      for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
        acc_merge(t, args.partials[((int64_t)by * gridDim.x + i) * kVals + v]);
      t = block_reduce<kBlock>(t);
      if (threadIdx.x == 0) {
        Acc run{args.acc[2 * s], args.acc[2 * s + 1]};
        acc_merge(run, t);
        args.acc[2 * s] = run.s;
        args.acc[2 * s + 1] = run.c;
      }
    }
    if (threadIdx.x == 0) *args.ticket = 0u;
  }
}

// Weighted sum of one integrand component (n_values == 1, the common case).
// Along a grid row every node shares its outer weight, so the kernels
// accumulate sum_j W_j f_j with the unscaled last-dimension weights W_j
// (fp64 values: one fused multiply-add per node; fp32 values: a compensated
// fp32 sum on the FP32 pipe) and fold the row's outer weight in once per row
// segment.  On GB300 an fp64 warp instruction holds a sub-partition's FP64
// unit for about 64 cycles, so fp64 sums are bound by the FP64 pipe near
// 0.75 of HBM bandwidth; fp32 sums by HBM.
template <typename F>
struct RowAcc;
template <>
struct RowAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double w, double v) { s = fma(w, v, s); }
  __device__ __forceinline__ double value() const { return s; }
  __device__ __forceinline__ void reset() { s = 0.0; }
};
template <>
struct RowAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float w, float v) {
    const float y = __fmaf_rn(w, v, -c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
  __device__ __forceinline__ void reset() { s = c = 0.f; }
};

template <typename F, int V>
__device__ __forceinline__ void load_vec(const F* __restrict__ p, F* v) {
  if constexpr (sizeof(F) == 8) {
    const double2 q = __ldg((const double2*)p);
    v[0] = q.x;
    v[1] = q.y;
  } else {
    const float4 q = __ldg((const float4*)p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  }
}

// Last-CTA reduction of the per-CTA partials into the running sum acc[0..1].
__device__ __forceinline__ void wsum_finish(const WsumArgs& args, Acc acc) {
  acc = block_reduce<kBlock>(acc);
  if (threadIdx.x == 0) args.partials[blockIdx.x] = acc;
  if (last_block_arrives(args.ticket)) {
    Acc t{0.0, 0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) acc_merge(t, args.partials[i]);
    t = block_reduce<kBlock>(t);
    if (threadIdx.x == 0) {
      Acc run{args.acc[0], args.acc[1]};
      acc_merge(run, t);
      args.acc[0] = run.s;
      args.acc[1] = run.c;
      *args.ticket = 0u;
    }
  }
}

// Short rows (n < 32): a thread walks strips of P consecutive nodes, read as
// 16-byte vectors when aligned, with the weights from a shared-memory table.
constexpr int kWTab = 4096;  // last-dimension weights a CTA keeps

template <typename T, typename D, bool GL, typename F, int P>
__global__ void __launch_bounds__(kBlock) weighted_sum1_kernel(WsumArgs args) {
  __shared__ Geo<T> g;
  __shared__ FastDiv fd_n;
  __shared__ F wt[kWTab];
  if (threadIdx.x == 0) {
    geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
    fd_n = make_fastdiv((uint32_t)args.n);
  }
  const int dim = args.dim, rule = args.rule, last = dim - 1;
  const int64_t n = args.n;
  const int n32 = (int)n;
  const bool tab = n <= kWTab;
  if (tab)
    for (int j = threadIdx.x; j < n32; j += blockDim.x) wt[j] = (F)wunit_at<GL>(rule, n, j, args.gl_weights);
  __syncthreads();
  const F* __restrict__ f = (const F*)args.f;
  constexpr int V = 16 / sizeof(F);  // values per 16-byte load
  const bool vec = (((uintptr_t)f) & 15) == 0;
  const bool small = (uint64_t)(args.start + args.count) <= 0xffffffffull;
  const double wlast = g.wscale[last];
  auto outer_w = [&](uint64_t row) -> double {
    double w = wlast;
    if (small) {
      uint32_t r = (uint32_t)row;
      for (int k = last - 1; k >= 0; --k) {
        const uint32_t q = fdiv(r, fd_n);
        w *= g.wscale[k] * wunit_at<GL>(rule, n, (int64_t)(r - q * fd_n.d), args.gl_weights);
        r = q;
      }
    } else {
      uint64_t r = row;
      for (int k = last - 1; k >= 0; --k) {
        const uint64_t q = r / (uint64_t)n;
        w *= g.wscale[k] * wunit_at<GL>(rule, n, (int64_t)(r - q * (uint64_t)n), args.gl_weights);
        r = q;
      }
    }
    return w;
  };
  Acc acc{0.0, 0.0};
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * P; base < args.count;
       base += nthreads * P) {
    const int cnt = (int)min((int64_t)P, args.count - base);
    const uint64_t node0 = (uint64_t)(args.start + base);
    uint64_t row;
    int j;
    if (small) {
      const uint32_t q = fdiv((uint32_t)node0, fd_n);
      row = q;
      j = (int)((uint32_t)node0 - q * fd_n.d);
    } else {
      row = node0 / (uint64_t)n;
      j = (int)(node0 - row * (uint64_t)n);
    }
    double w_outer = outer_w(row);
    RowAcc<F> ra;
#pragma unroll
    for (int i0 = 0; i0 < P; i0 += V) {
      F v[V];
      if (vec && i0 + V <= cnt) {
        load_vec<F, V>(f + base + i0, v);
      } else {
#pragma unroll
        for (int q = 0; q < V; ++q) v[q] = i0 + q < cnt ? __ldg(f + base + i0 + q) : (F)0;
      }
#pragma unroll
      for (int q = 0; q < V; ++q) {
        if (i0 + q < cnt) {
          ra.add(tab ? wt[j] : (F)wunit_at<GL>(rule, n, j, args.gl_weights), v[q]);
          if (++j == n32 && i0 + q + 1 < cnt) {  // the strip enters the next row
            acc_add(acc, ra.value() * w_outer);
            ra.reset();
            j = 0;
            w_outer = outer_w(++row);
          }
        }
      }
    }
    acc_add(acc, ra.value() * w_outer);
  }
  wsum_finish(args, acc);
}

// Rows of at least 32 nodes: a warp takes whole grid rows, its lanes read
// the row with coalesced loads and accumulate W_j f_j, and each lane folds
// the row's outer weight in once per row (products of per-dimension weight
// tables in shared memory).  Rows cut by the chunk's start or end are
// summed over their part in the chunk.
constexpr int kRowTab = 2048;  // entries of each weight table

template <typename T, typename D, bool GL, typename F>
__global__ void __launch_bounds__(kBlock) weighted_sum_rows_kernel(WsumArgs args) {
  __shared__ Geo<T> g;
  __shared__ FastDiv fd_n;
  __shared__ F wl[kRowTab];       // unscaled last-dimension weights
  __shared__ double wo[kRowTab];  // wo[k*n + j] = wscale_k * W_k(j), outer dimensions k
  if (threadIdx.x == 0) {
    geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
    fd_n = make_fastdiv((uint32_t)args.n);
  }
  __syncthreads();
  const int dim = args.dim, rule = args.rule, last = dim - 1;
  const int64_t n = args.n;
  const int n32 = (int)n;
  for (int j = threadIdx.x; j < n32; j += blockDim.x) wl[j] = (F)wunit_at<GL>(rule, n, j, args.gl_weights);
  for (int e = threadIdx.x; e < last * n32; e += blockDim.x) {
    const int k = e / n32;
    wo[e] = g.wscale[k] * wunit_at<GL>(rule, n, e - k * n32, args.gl_weights);
  }
  __syncthreads();
  const F* __restrict__ f = (const F*)args.f;
  const int lane = threadIdx.x & 31;
  const int64_t end = args.start + args.count;
  const uint64_t row_begin = (uint64_t)args.start / (uint64_t)n;
  const uint64_t row_end = ((uint64_t)end + (uint64_t)n - 1) / (uint64_t)n;
  const bool small = (uint64_t)end <= 0xffffffffull;
  const double wlast = g.wscale[last];
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  double lane_acc = 0.0;
  for (uint64_t r = row_begin + (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < row_end;
       r += (uint64_t)nwarps) {
    double w = wlast;
    if (small) {
      uint32_t q = (uint32_t)r;
      for (int k = last - 1; k >= 0; --k) {
        const uint32_t q2 = fdiv(q, fd_n);
        w *= wo[k * n32 + (int)(q - q2 * fd_n.d)];
        q = q2;
      }
    } else {
      uint64_t q = r;
      for (int k = last - 1; k >= 0; --k) {
        const uint64_t q2 = q / (uint64_t)n;
        w *= wo[k * n32 + (int)(q - q2 * (uint64_t)n)];
        q = q2;
      }
    }
    const int64_t r0 = (int64_t)r * n;
    const int j0 = (int)max((int64_t)0, args.start - r0);
    const int j1 = (int)min(n, end - r0);
    const F* fr = f + (r0 - args.start);
    RowAcc<F> ra;
#pragma unroll 4
    for (int j = j0 + lane; j < j1; j += 32) ra.add(wl[j], __ldg(fr + j));
    lane_acc += ra.value() * w;
  }
  wsum_finish(args, Acc{lane_acc, 0.0});
}

// fp64 values, rows of at least 32 nodes: the walk of weighted_sum_rows_kernel
// with every product and sum as a double-float on the FP32 pipe.  A value is
// split into two floats by integer operations (f2_split: 47 of its 53
// significant bits, rounded); the weights are double-float tables
// (Newton-Cotes unit weights are small integers, exact in one float).  On
// GB300 the FP64 unit is the limit of one fp64 fused multiply-add per value
// (FP64 pipe 82 % active, a quarter of HBM bandwidth); this form issues
// about 75 instructions per value on the other pipes and is 19 % faster.
// Each term is within about 2^-46 of w_i f_i and the sums are double-floats,
// an error bound of the order of an fp64 pairwise sum's.  The float range
// bounds where this holds: values outside 2^-40 <= |f| < 2^40 (and
// subnormal, infinite, NaN ones) go to an fp64 side sum, and a grid whose
// node weights leave [2^-40, 2^40] is summed in fp64 throughout.  The CTA's
// sum becomes fp64 once, in thread 0.
template <typename T, typename D, bool GL>
__global__ void __launch_bounds__(kBlock) weighted_sum_rows_f2_kernel(WsumArgs args) {
  __shared__ Geo<T> g;
  __shared__ FastDiv fd_n;
  __shared__ F2 wl[kRowTab];  // unscaled last-dimension weights
  __shared__ F2 wo[kRowTab];  // wo[k*n + j] = wscale_k * W_k(j), outer dimensions k
  __shared__ F2 ws[kMaxDim];
  __shared__ F2 red[kBlock / 32];
  __shared__ unsigned umin_bits, umax_bits;  // extreme |unit weight| (Gauss), as float bits
  __shared__ int use_f2;
  if (threadIdx.x == 0) {
    geo_setup<T, D>(g, args.rule, args.dim, args.n, (const D*)args.domain);
    fd_n = make_fastdiv((uint32_t)args.n);
    umin_bits = 0x7f7fffffu;
    umax_bits = 0u;
  }
  __syncthreads();
  const int dim = args.dim, rule = args.rule, last = dim - 1;
  const int64_t n = args.n;
  const int n32 = (int)n;
  if (threadIdx.x < dim) ws[threadIdx.x] = f2_from_double(g.wscale[threadIdx.x]);
  for (int j = threadIdx.x; j < n32; j += blockDim.x) {
    if (GL) {
      const double u = __ldg(args.gl_weights + j);
      wl[j] = f2_from_double(u);
      const unsigned ub = __float_as_uint(fabsf((float)u));  // positive floats order as integers
      atomicMin(&umin_bits, ub);
      atomicMax(&umax_bits, ub);
    } else {
      wl[j] = F2{(float)nc_int(rule, j, n), 0.f};
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // bounds of every node weight: prod_k |wscale_k| x (largest | smallest unit weight)
    const double umax = GL ? (double)__uint_as_float(umax_bits)
                           : (rule == TQ_RULE_TRAPEZOID ? 2.0 : (rule == TQ_RULE_SIMPSON ? 4.0 : 32.0));
    const double umin = GL ? (double)__uint_as_float(umin_bits) : 1.0;
    double hi = 1.0, lo = 1.0;
    for (int k = 0; k < dim; ++k) {
      hi *= fabs(g.wscale[k]) * umax;
      lo *= fabs(g.wscale[k]) * umin;
    }
    use_f2 = hi <= 0x1p40 && lo >= 0x1p-40;  // false for NaN
  }
  for (int e = threadIdx.x; e < last * n32; e += blockDim.x) {
    const int k = e / n32;
    wo[e] = f2_mul(ws[k], wl[e - k * n32]);
  }
  __syncthreads();
  const double* __restrict__ f = (const double*)args.f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t end = args.start + args.count;
  const uint64_t row_begin = (uint64_t)args.start / (uint64_t)n;
  const uint64_t row_end = ((uint64_t)end + (uint64_t)n - 1) / (uint64_t)n;
  const bool small = (uint64_t)end <= 0xffffffffull;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t r_first = row_begin + (uint64_t)blockIdx.x * (blockDim.x >> 5) + (uint64_t)warp;
  Acc acc{0.0, 0.0};
  if (!use_f2) {
    // node weights outside the double-float range: fp64 throughout
    double lane_d = 0.0;
    for (uint64_t r = r_first; r < row_end; r += (uint64_t)nwarps) {
      double w = g.wscale[last];
      uint64_t q = r;
      for (int k = last - 1; k >= 0; --k) {
        const uint64_t q2 = q / (uint64_t)n;
        w *= g.wscale[k] * wunit_at<GL>(rule, n, (int64_t)(q - q2 * (uint64_t)n), args.gl_weights);
        q = q2;
      }
      const int64_t r0 = (int64_t)r * n;
      const int j0 = (int)max((int64_t)0, args.start - r0);
      const int j1 = (int)min(n, end - r0);
      const double* fr = f + (r0 - args.start);
      double rsum = 0.0;
      for (int j = j0 + lane; j < j1; j += 32)
        rsum = fma(wunit_at<GL>(rule, n, j, args.gl_weights), __ldg(fr + j), rsum);
      lane_d = fma(rsum, w, lane_d);
    }
    acc = block_reduce<kBlock>(Acc{lane_d, 0.0});
  } else {
    F2 lane_acc{0.f, 0.f};
    double side = 0.0;  // fp64 sum of the values f2_split leaves out
    int any_side = 0;
    for (uint64_t r = r_first; r < row_end; r += (uint64_t)nwarps) {
      F2 w = ws[last];
      if (small) {
        uint32_t q = (uint32_t)r;
        for (int k = last - 1; k >= 0; --k) {
          const uint32_t q2 = fdiv(q, fd_n);
          w = f2_mul(w, wo[k * n32 + (int)(q - q2 * fd_n.d)]);
          q = q2;
        }
      } else {
        uint64_t q = r;
        for (int k = last - 1; k >= 0; --k) {
          const uint64_t q2 = q / (uint64_t)n;
          w = f2_mul(w, wo[k * n32 + (int)(q - q2 * (uint64_t)n)]);
          q = q2;
        }
      }
      const int64_t r0 = (int64_t)r * n;
      const int j0 = (int)max((int64_t)0, args.start - r0);
      const int j1 = (int)min(n, end - r0);
      const double* fr = f + (r0 - args.start);
      float sh = 0.f, sl = 0.f;  // the lane's row sum, hi + lo (lo unnormalised)
      double rs = 0.0;
      bool rside = false;
      // four loads in flight per lane, then their sums
      for (int jb = j0 + lane; jb < j1; jb += 128) {
        double x[4];
        int jj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = jb + 32 * u;
          jj[u] = j < j1 ? j : j0;
          x[u] = j < j1 ? __ldg(fr + j) : 0.0;
        }
        unsigned side_mask = 0u;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const F2Split v = f2_split(x[u]);
          side_mask |= (unsigned)(!v.ok) << u;
          const F2 wj = wl[jj[u]];
          const float p = __fmul_rn(wj.hi, v.v.hi);  // w_j f_j = p + e, e to about 2^-46
          float e = __fmaf_rn(wj.hi, v.v.hi, -p);
          e = __fmaf_rn(wj.hi, v.v.lo, e);
          if (GL) e = __fmaf_rn(wj.lo, v.v.hi, e);
          const F2 t = two_sum(sh, p);
          sh = t.hi;
          sl = __fadd_rn(sl, __fadd_rn(t.lo, e));
        }
        if (side_mask) {  // the rare values outside the split's range
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if ((side_mask >> u) & 1u) {
              rs = fma(f2_value(wl[jj[u]]), x[u], rs);
              rside = true;
            }
        }
      }
      lane_acc = f2_add(lane_acc, f2_mul(two_sum(sh, sl), w));
      if (rside) {
        side = fma(rs, f2_value(w), side);
        any_side = 1;
      }
    }
    // the CTA's double-float sum in a fixed tree; fp64 once per CTA
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lane_acc = f2_add(lane_acc, f2_shfl_down(lane_acc, o));
    if (lane == 0) red[warp] = lane_acc;
    const bool cta_side = __syncthreads_or(any_side) != 0;
    if (warp == 0) {
      F2 t = lane < kBlock / 32 ? red[lane] : F2{0.f, 0.f};
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t = f2_add(t, f2_shfl_down(t, o));
      if (lane == 0) {
        acc_add(acc, (double)t.hi);
        acc_add(acc, (double)t.lo);
      }
    }
    if (cta_side) {  // rare: the side sums in fp64
      const Acc sa = block_reduce<kBlock>(Acc{side, 0.0});
      if (threadIdx.x == 0) acc_merge(acc, sa);
    }
  }
  if (threadIdx.x == 0) args.partials[blockIdx.x] = acc;
  if (last_block_arrives(args.ticket)) {
    Acc t{0.0, 0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) acc_merge(t, args.partials[i]);
    t = block_reduce<kBlock>(t);
    if (threadIdx.x == 0) {
      Acc run{args.acc[0], args.acc[1]};
      acc_merge(run, t);
      args.acc[0] = run.s;
      args.acc[1] = run.c;
      *args.ticket = 0u;
    }
  }
}

template <typename D>
__global__ void finalize_kernel(int rule, int dim, const D* __restrict__ dom, int64_t npts,
                                const double* __restrict__ acc, int64_t S, void* out,
                                int out_dtype) {
  double scale = 1.0;
  if (rule == TQ_RULE_MC) {
    // monte_carlo.py:72-77: volume = prod(b - a) in the domain type
    D vol = (D)1;
    for (int k = 0; k < dim; ++k) vol = vol * (D)(dom[2 * k + 1] - dom[2 * k]);
    scale = (double)vol / (double)npts;
  }
  for (int64_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
    const double v = scale * (acc[2 * s] + acc[2 * s + 1]);
    if (out_dtype == TQ_F64)
      ((double*)out)[s] = v;
    else
      ((float*)out)[s] = (float)v;
  }
}

}  // namespace tq

using namespace tq;

// --------------------------------------------------------------- C ABI
static bool valid_rule(int rule, int64_t n) {
  switch (rule) {
    case TQ_RULE_TRAPEZOID:
    case TQ_RULE_GAUSS:
      return n >= 2;
    case TQ_RULE_SIMPSON:
      return n >= 3 && (n & 1) == 1;
    case TQ_RULE_BOOLE:
      return n >= 5 && (n - 1) % 4 == 0;
    default:
      return false;
  }
}

static bool grid_total(int dim, int64_t n, int64_t* total) {
  int64_t t = 1;
  for (int k = 0; k < dim; ++k) {
    if (t > (int64_t(1) << 62) / n) return false;
    t *= n;
  }
  *total = t;
  return true;
}

static constexpr int kStripF = 32, kStripD = 16;

static int64_t fused_blocks(int64_t total, int strip) {
  const int64_t need = (total + (int64_t)kBlock * strip - 1) / ((int64_t)kBlock * strip);
  const int64_t cap = (int64_t)sm_count() * 8;
  return need < 1 ? 1 : (need < cap ? need : cap);
}

extern "C" size_t tq_grid_fused_workspace_size(int rule, int dim, int64_t n_per_dim) {
  (void)rule;
  (void)dim;
  (void)n_per_dim;
  return reduce_ws_bytes((int64_t)sm_count() * 8);
}

extern "C" int tq_grid_fused(int dtype, int rule, int dim, int64_t n_per_dim, const void* domain,
                             const double* gl_nodes, const double* gl_weights, int family,
                             const double* params, void* out, int out_dtype, double* out64,
                             void* workspace, size_t workspace_bytes, void* stream) {
  if (!valid_dtype(dtype) || !valid_dtype(out_dtype)) return TQ_ERR_DTYPE;
  if (dim < 1 || dim > kMaxDim) return TQ_ERR_DIM;
  if (!valid_rule(rule, n_per_dim)) return TQ_ERR_RULE;
  if (!domain || !params || !workspace || (!out && !out64)) return TQ_ERR_ARG;
  if (rule == TQ_RULE_GAUSS && (!gl_nodes || !gl_weights)) return TQ_ERR_ARG;
  int64_t total;
  if (!grid_total(dim, n_per_dim, &total)) return TQ_ERR_TOO_LARGE;
  const bool gl = rule == TQ_RULE_GAUSS;
  const bool f64 = gl || dtype == TQ_F64;
  const int64_t blocks = fused_blocks(total, f64 ? kStripD : kStripF);
  if (workspace_bytes < reduce_ws_bytes(blocks)) return TQ_ERR_WORKSPACE;
  FusedArgs a;
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
  a.partials = (Acc*)((char*)workspace + 256);
  a.out = out;
  a.out_dtype = out_dtype;
  a.out64 = out64;
  cudaStream_t s = (cudaStream_t)stream;
  const dim3 grid((unsigned)blocks);
#define TQ_FUSED_RULE(RULEC)                                                              \
  if (gl) {                                                                                \
    if (dtype == TQ_F64)                                                                   \
      grid_fused_kernel<double, double, RULEC, FAM, kStripD><<<grid, kBlock, 0, s>>>(a);   \
    else                                                                                   \
      grid_fused_kernel<double, float, RULEC, FAM, kStripD><<<grid, kBlock, 0, s>>>(a);    \
  } else if (dtype == TQ_F64) {                                                            \
    grid_fused_kernel<double, double, RULEC, FAM, kStripD><<<grid, kBlock, 0, s>>>(a);     \
  } else {                                                                                 \
    grid_fused_kernel<float, float, RULEC, FAM, kStripF><<<grid, kBlock, 0, s>>>(a);       \
  }
  TQ_DISPATCH_FAMILY(family, FAM, {
    switch (rule) {
      case TQ_RULE_TRAPEZOID: { TQ_FUSED_RULE(TQ_RULE_TRAPEZOID) } break;
      case TQ_RULE_SIMPSON: { TQ_FUSED_RULE(TQ_RULE_SIMPSON) } break;
      case TQ_RULE_BOOLE: { TQ_FUSED_RULE(TQ_RULE_BOOLE) } break;
      default: {
        if (dtype == TQ_F64)
          grid_fused_kernel<double, double, TQ_RULE_GAUSS, FAM, kStripD><<<grid, kBlock, 0, s>>>(a);
        else
          grid_fused_kernel<double, float, TQ_RULE_GAUSS, FAM, kStripD><<<grid, kBlock, 0, s>>>(a);
      }
    }
  });
#undef TQ_FUSED_RULE
  return launch_status();
}

static int64_t stream_blocks(int64_t work) {
  const int64_t need = (work + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)sm_count() * 16;
  return need < 1 ? 1 : (need < cap ? need : cap);
}

extern "C" int tq_grid_points(int dtype, int rule, int dim, int64_t n_per_dim,
                              const void* domain, const double* gl_nodes, int64_t start,
                              int64_t count, void* points, void* stream) {
  if (!valid_dtype(dtype)) return TQ_ERR_DTYPE;
  if (dim < 1 || dim > kMaxDim) return TQ_ERR_DIM;
  if (!valid_rule(rule, n_per_dim)) return TQ_ERR_RULE;
  if (!domain || !points || start < 0 || count < 0) return TQ_ERR_ARG;
  if (rule == TQ_RULE_GAUSS && !gl_nodes) return TQ_ERR_ARG;
  int64_t total;
  if (!grid_total(dim, n_per_dim, &total)) return TQ_ERR_TOO_LARGE;
  if (start + count > total) return TQ_ERR_ARG;
  if (count == 0) return TQ_OK;
  PointsArgs a{rule, dim, n_per_dim, start, count, domain, gl_nodes, points};
  cudaStream_t s = (cudaStream_t)stream;
  const size_t tsize = (rule == TQ_RULE_GAUSS || dtype == TQ_F64) ? 8 : 4;
  // tiles of a multiple of 16 points that fill a 24 KiB buffer
  const int tile_pts = (int)((kPtsTileBytes / (tsize * (size_t)dim)) & ~(size_t)15);
  if ((((uintptr_t)points) & 15) == 0 && tile_pts >= 16) {
    const int64_t n_tiles = (count + tile_pts - 1) / tile_pts;
    const int64_t cap = (int64_t)sm_count() * 4;
    const dim3 grid((unsigned)(n_tiles < cap ? n_tiles : cap));
    const size_t smem = 2 * (size_t)kPtsTileBytes;
#define TQ_PTS_TILED(T, D, GLB)                                                                     \
  {                                                                                                 \
    auto k = grid_points_tiled_kernel<T, D, GLB>;                                                   \
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e != cudaSuccess) return set_cuda_error(e);                                                 \
    k<<<grid, kBlock, smem, s>>>(a, tile_pts, n_tiles);                                             \
  }
    if (rule == TQ_RULE_GAUSS) {
      if (dtype == TQ_F64) TQ_PTS_TILED(double, double, true)
      else TQ_PTS_TILED(double, float, true)
    } else if (dtype == TQ_F64) {
      TQ_PTS_TILED(double, double, false)
    } else {
      TQ_PTS_TILED(float, float, false)
    }
#undef TQ_PTS_TILED
    return launch_status();
  }
  // unaligned output: one thread per element
  const dim3 grid((unsigned)stream_blocks(count * dim));
  if (rule == TQ_RULE_GAUSS) {
    if (dtype == TQ_F64)
      grid_points_kernel<double, double, true><<<grid, kBlock, 0, s>>>(a);
    else
      grid_points_kernel<double, float, true><<<grid, kBlock, 0, s>>>(a);
  } else if (dtype == TQ_F64) {
    grid_points_kernel<double, double, false><<<grid, kBlock, 0, s>>>(a);
  } else {
    grid_points_kernel<float, float, false><<<grid, kBlock, 0, s>>>(a);
  }
  return launch_status();
}

extern "C" int tq_grid_weights(int dtype, int rule, int dim, int64_t n_per_dim,
                               const void* domain, const double* gl_weights, int64_t start,
                               int64_t count, double* weights, void* stream) {
  if (!valid_dtype(dtype)) return TQ_ERR_DTYPE;
  if (dim < 1 || dim > kMaxDim) return TQ_ERR_DIM;
  if (!valid_rule(rule, n_per_dim)) return TQ_ERR_RULE;
  if (!domain || !weights || start < 0 || count < 0) return TQ_ERR_ARG;
  if (rule == TQ_RULE_GAUSS && !gl_weights) return TQ_ERR_ARG;
  int64_t total;
  if (!grid_total(dim, n_per_dim, &total)) return TQ_ERR_TOO_LARGE;
  if (start + count > total) return TQ_ERR_ARG;
  if (count == 0) return TQ_OK;
  WeightsArgs a{rule, dim, n_per_dim, start, count, domain, gl_weights, weights};
  cudaStream_t s = (cudaStream_t)stream;
  const dim3 grid((unsigned)stream_blocks(count));
  if (rule == TQ_RULE_GAUSS) {
    if (dtype == TQ_F64)
      grid_weights_kernel<double, double, true><<<grid, kBlock, 0, s>>>(a);
    else
      grid_weights_kernel<double, float, true><<<grid, kBlock, 0, s>>>(a);
  } else if (dtype == TQ_F64) {
    grid_weights_kernel<double, double, false><<<grid, kBlock, 0, s>>>(a);
  } else {
    grid_weights_kernel<float, float, false><<<grid, kBlock, 0, s>>>(a);
  }
  return launch_status();
}

static constexpr int kStripW = 8;
static constexpr int kStripW1 = 32;  // nodes per strip of the short-row weighted sum

static int64_t wsum_blocks_x(int64_t count) {
  const int64_t need = (count + (int64_t)kBlock * kStripW - 1) / ((int64_t)kBlock * kStripW);
  const int64_t cap = (int64_t)sm_count() * 8;
  return need < 1 ? 1 : (need < cap ? need : cap);
}

extern "C" size_t tq_weighted_sum_workspace_size(int64_t count, int64_t n_values) {
  const int64_t gy = (n_values + kVals - 1) / kVals;
  return reduce_ws_bytes(wsum_blocks_x(count) * gy * kVals);
}

extern "C" int tq_weighted_sum(int dtype, int rule, int dim, int64_t n_per_dim,
                               const void* domain, const double* gl_weights, int64_t start,
                               int64_t count, const void* f, int f_dtype, int64_t n_values,
                               double* acc, void* workspace, size_t workspace_bytes,
                               void* stream) {
  if (!valid_dtype(dtype) || !valid_dtype(f_dtype)) return TQ_ERR_DTYPE;
  if (dim < 1 || dim > kMaxDim) return TQ_ERR_DIM;
  if (rule != TQ_RULE_MC && !valid_rule(rule, n_per_dim)) return TQ_ERR_RULE;
  if (!domain || !f || !acc || !workspace || start < 0 || count < 0 || n_values < 1)
    return TQ_ERR_ARG;
  if (rule == TQ_RULE_GAUSS && !gl_weights) return TQ_ERR_ARG;
  if (rule != TQ_RULE_MC) {
    int64_t total;
    if (!grid_total(dim, n_per_dim, &total)) return TQ_ERR_TOO_LARGE;
    if (start + count > total) return TQ_ERR_ARG;
  }
  if (count == 0) return TQ_OK;
  const int64_t gy = (n_values + kVals - 1) / kVals;
  if (gy > 65535) return TQ_ERR_TOO_LARGE;
  const int64_t gx = wsum_blocks_x(count);
  if (workspace_bytes < reduce_ws_bytes(gx * gy * kVals)) return TQ_ERR_WORKSPACE;
  WsumArgs a;
  a.rule = rule;
  a.dim = dim;
  a.n = n_per_dim;
  a.start = start;
  a.count = count;
  a.n_values = n_values;
  a.domain = domain;
  a.gl_weights = gl_weights;
  a.f = f;
  a.acc = acc;
  a.ticket = (unsigned*)workspace;
  a.partials = (Acc*)((char*)workspace + 256);
  cudaStream_t s = (cudaStream_t)stream;
  const dim3 grid((unsigned)gx, (unsigned)gy);
  const bool gl = rule == TQ_RULE_GAUSS;
  // one component of a grid rule: the row kernels (row weights, coalesced
  // or vector loads); Monte Carlo and vector integrands: the general one
  const bool scalar = n_values == 1 && rule != TQ_RULE_MC;
  const bool rows = scalar && n_per_dim >= 32 && n_per_dim <= kRowTab && (dim - 1) * n_per_dim <= kRowTab;
  int64_t g1 = (count + (int64_t)kBlock * kStripW1 - 1) / ((int64_t)kBlock * kStripW1);
  g1 = g1 < 1 ? 1 : (g1 < gx ? g1 : gx);  // the workspace holds gx partials
  const dim3 grid1((unsigned)g1);
#define TQ_WSUM(T, D, GLB)                                                                   \
  if (rows) {                                                                                \
    if (f_dtype == TQ_F64)                                                                   \
      weighted_sum_rows_f2_kernel<T, D, GLB><<<grid, kBlock, 0, s>>>(a);                     \
    else                                                                                     \
      weighted_sum_rows_kernel<T, D, GLB, float><<<grid, kBlock, 0, s>>>(a);                 \
  } else if (scalar) {                                                                       \
    if (f_dtype == TQ_F64)                                                                   \
      weighted_sum1_kernel<T, D, GLB, double, kStripW1><<<grid1, kBlock, 0, s>>>(a);         \
    else                                                                                     \
      weighted_sum1_kernel<T, D, GLB, float, kStripW1><<<grid1, kBlock, 0, s>>>(a);          \
  } else if (f_dtype == TQ_F64) {                                                            \
    weighted_sum_kernel<T, D, GLB, double, kStripW><<<grid, kBlock, 0, s>>>(a);              \
  } else {                                                                                   \
    weighted_sum_kernel<T, D, GLB, float, kStripW><<<grid, kBlock, 0, s>>>(a);               \
  }
  if (gl) {
    if (dtype == TQ_F64) {
      TQ_WSUM(double, double, true)
    } else {
      TQ_WSUM(double, float, true)
    }
  } else if (dtype == TQ_F64) {
    TQ_WSUM(double, double, false)
  } else {
    TQ_WSUM(float, float, false)
  }
#undef TQ_WSUM
  return launch_status();
}

extern "C" int tq_finalize_sum(int dtype, int rule, int dim, const void* domain, int64_t n_points,
                               const double* acc, int64_t n_values, void* out, int out_dtype,
                               void* stream) {
  if (!valid_dtype(dtype) || !valid_dtype(out_dtype)) return TQ_ERR_DTYPE;
  if (dim < 1) return TQ_ERR_DIM;
  if (!domain || !acc || !out || n_values < 1 || n_points < 1) return TQ_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((n_values + kBlock - 1) / kBlock);
  if (dtype == TQ_F64)
    finalize_kernel<double><<<blocks, kBlock, 0, s>>>(rule, dim, (const double*)domain, n_points,
                                                      acc, n_values, out, out_dtype);
  else
    finalize_kernel<float><<<blocks, kBlock, 0, s>>>(rule, dim, (const float*)domain, n_points,
                                                     acc, n_values, out, out_dtype);
  return launch_status();
}

// ------------------------------------------- allocation-free entry point
// For callers that cannot allocate device memory at call time: a plugin
// inside a host application that owns all device memory, code that must not
// allocate once it runs (a fixed-latency loop), or a plain C caller that has
// no allocator to hand.  The CTA partials and the ticket word of the fused
// grid rule live in this file-scope device array instead of a caller-given
// workspace.  Every GPU that loads the library holds it until exit.
#include <mutex>

namespace {

constexpr int kNoAllocSlots = 4096;  // CTA partials the static scratch holds
constexpr size_t kNoAllocBytes = 256 + (size_t)kNoAllocSlots * sizeof(tq::Acc);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (host code only sees a host-side stand-in under the array's
// name, which must never be handed to a kernel).
int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return tq::set_cuda_error(e);
  if (dev < 0 || dev >= 64) return TQ_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return tq::set_cuda_error(e == cudaSuccess ? cudaErrorInvalidSymbol : e);
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return TQ_OK;
}

}  // namespace

extern "C" int tq_grid_fused_noalloc(int dtype, int rule, int dim, int64_t n_per_dim,
                                     const void* domain, const double* gl_nodes,
                                     const double* gl_weights, int family, const double* params,
                                     void* out, int out_dtype, double* out64, void* stream) {
  if (tq_grid_fused_workspace_size(rule, dim, n_per_dim) > kNoAllocBytes) return TQ_ERR_SCRATCH;
  void* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != TQ_OK) return rc;
  // the ticket word must start at zero; the last CTA leaves it at zero
  const cudaError_t e = cudaMemsetAsync(scratch, 0, 16, (cudaStream_t)stream);
  if (e != cudaSuccess) return tq::set_cuda_error(e);
  return tq_grid_fused(dtype, rule, dim, n_per_dim, domain, gl_nodes, gl_weights, family, params,
                       out, out_dtype, out64, scratch, kNoAllocBytes, stream);
}
