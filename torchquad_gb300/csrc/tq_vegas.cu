// VEGAS+ on GB300: the stratification update (get_NH), the end of an
// iteration (estimate, variance and update_DH), the adaptive-map update, and
// the C-ABI entry points of the VEGAS state.  The fused sampler is in
// tq_vegas_sample.cuh.
//
// Reference (torchquad v0.5.0): vegas.py (driver), vegas_map.py (adaptive
// map), vegas_stratification.py (stratified sampling).

#include <type_traits>

#include "tq_vegas_sample.cuh"

namespace tq {

// ----------------------------------------------------------- get_NH
struct NhArgs {
  tq_vegas_state st;
  int64_t* block_tot;  // [blocks]
  unsigned* ticket;
  int split;  // leave cube_start block-local (see kCtlSplit)
};

template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_nh_kernel(NhArgs a) {
  const tq_vegas_state& st = a.st;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nh = 0;
  const int64_t nevals_exp = st.control[0];
  const int64_t normalize = st.control[2];
  if (c < st.n_cubes) {
    T dh = ((T*)st.dh)[c];
    if (normalize) {
      const T sum = (T)st.scalars[0];
      if (sum != (T)0) {
        dh = div_rn(dh, sum);  // vegas_stratification.py:88-90
        ((T*)st.dh)[c] = dh;
      }
    }
    T f = floor(mul_rn(dh, (T)nevals_exp));  // :102
    f = f < (T)2 ? (T)2 : f;                    // :103 clip(nh, 2, None)
    nh = (int64_t)f;
    st.neval[c] = nh;
    st.jf[c] = 0.0;
    st.jf2[c] = 0.0;
  }
  // block-wide exclusive scan of nh (deterministic)
  __shared__ int64_t warp_tot[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t incl = nh;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < kBlock / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t v = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += v;
    }
    if (lane < kBlock / 32) warp_tot[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const int64_t excl = incl - nh + (warp > 0 ? warp_tot[warp - 1] : 0);
  if (c < st.n_cubes) st.cube_start[c] = excl;
  if (threadIdx.x == 0) a.block_tot[blockIdx.x] = warp_tot[kBlock / 32 - 1];
  if (last_block_arrives(a.ticket)) {
    // exclusive scan of the block totals, kBlock at a time
    int64_t carry = 0;
    for (unsigned base = 0; base < gridDim.x; base += kBlock) {
      const unsigned b = base + threadIdx.x;
      const int64_t t = b < gridDim.x ? a.block_tot[b] : 0;
      int64_t x = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t v = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += v;
      }
      __syncthreads();
      if (lane == 31) warp_tot[warp] = x;
      __syncthreads();
      if (warp == 0) {
        int64_t w = lane < kBlock / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int64_t v = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += v;
        }
        if (lane < kBlock / 32) warp_tot[lane] = w;
      }
      __syncthreads();
      const int64_t ex = carry + x - t + (warp > 0 ? warp_tot[warp - 1] : 0);
      if (b < gridDim.x) a.block_tot[b] = ex;
      carry += warp_tot[kBlock / 32 - 1];
    }
    if (threadIdx.x == 0) {
      st.cube_start[st.n_cubes] = carry;
      st.control[2] = 0;
      st.control[kCtlSplit] = a.split;
      *a.ticket = 0u;
    }
  }
}

__global__ void __launch_bounds__(kBlock) vegas_nh_fixup_kernel(tq_vegas_state st,
                                                                const int64_t* block_pre) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < st.n_cubes) st.cube_start[c] += block_pre[blockIdx.x];
}

// ---------------------------------------------------- finish iteration
struct FinishArgs {
  tq_vegas_state st;
  double beta;
  double V;       // V_cubes = (1/n_strat)^dim, computed on the host
  Acc* partials;  // [blocks][3]
  unsigned* ticket;
  const int64_t* block_pre;  // block offsets of a split cube_start (kCtlSplit)
};

// Three plain fp64 tree sums over the CTA at once (pairwise: error O(log n)
// ulp; the three chains interleave); results valid in thread 0.  The
// compensated sum is taken across CTAs by the last one.
__device__ __forceinline__ void block_sum3(double& x, double& y, double& z, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    x += __shfl_down_sync(0xffffffffu, x, o);
    y += __shfl_down_sync(0xffffffffu, y, o);
    z += __shfl_down_sync(0xffffffffu, z, o);
  }
  if (lane == 0) {
    sh[warp] = x;
    sh[32 + warp] = y;
    sh[64 + warp] = z;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    x = lane < nw ? sh[lane] : 0.0;
    y = lane < nw ? sh[32 + lane] : 0.0;
    z = lane < nw ? sh[64 + lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_down_sync(0xffffffffu, x, o);
      y += __shfl_down_sync(0xffffffffu, y, o);
      z += __shfl_down_sync(0xffffffffu, z, o);
    }
  }
}

template <typename T>
__device__ void finish_body(const FinishArgs& a, unsigned bid, unsigned nblk) {
  __shared__ double sh[96];
  const tq_vegas_state& st = a.st;
  const double V = a.V;  // V_cubes (vegas_stratification.py:29)
  const T Vt = (T)V, V2t = (T)(V * V);
  const T beta = (T)a.beta;
  double res = 0.0, s2 = 0.0, dsum = 0.0;
  const bool split = st.control[kCtlSplit] != 0;
  for (int64_t c = (int64_t)bid * blockDim.x + threadIdx.x; c < st.n_cubes;
       c += (int64_t)nblk * blockDim.x) {
    if (split) st.cube_start[c] += a.block_pre[c / kBlock];
    const int64_t nn = st.neval[c];
    const double J = st.jf[c], J2 = st.jf2[c];
    const double inv = 1.0 / (double)nn;
    const double ih = J * (inv * V);                           // vegas.py:294
    res += ih;
    s2 += fabs(J2 * inv * (V * V) - ih * ih) * inv;            // :297-303
    // update_DH (vegas_stratification.py:72-86) in the state's dtype
    const T cnt = (T)nn, jT = (T)J, j2T = (T)J2;
    const T q = div_rn(mul_rn(Vt, jT), cnt);
    T dt = sub_rn(div_rn(mul_rn(V2t, j2T), cnt), mul_rn(q, q));
    if (dt < (T)0) dt = (T)0;
    const T dh = (a.beta == 0.75) ? pow(dt, (T)0.75) : pow(dt, beta);
    ((T*)st.dh)[c] = dh;
    dsum += (double)dh;
  }
  block_sum3(res, s2, dsum, sh);
  if (threadIdx.x == 0) {
    a.partials[3 * bid] = Acc{res, 0.0};
    a.partials[3 * bid + 1] = Acc{s2, 0.0};
    a.partials[3 * bid + 2] = Acc{dsum, 0.0};
  }
  if (last_block_of(a.ticket, nblk) && threadIdx.x < 32) {
    // one warp, fixed assignment of partials to lanes and a fixed tree:
    // deterministic; the three compensated chains interleave
    const int lane = threadIdx.x;
    Acc r{0, 0}, q{0, 0}, ds{0, 0};
    for (unsigned i = lane; i < nblk; i += 32) {
      acc_add(r, __ldcg(&a.partials[3 * i].s));
      acc_add(q, __ldcg(&a.partials[3 * i + 1].s));
      acc_add(ds, __ldcg(&a.partials[3 * i + 2].s));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const Acc r2 = acc_shfl_down(r, off), q2 = acc_shfl_down(q, off), d2 = acc_shfl_down(ds, off);
      acc_merge(r, r2);
      acc_merge(q, q2);
      acc_merge(ds, d2);
    }
    if (lane == 0) {
      const int64_t slot = st.control[1];
      if (slot >= 0 && slot < st.n_stat_slots) {
        double* out = st.stats + 4 * slot;
        out[0] = r.s + r.c;
        out[1] = q.s + q.c;
        out[2] = (double)st.cube_start[st.n_cubes];
      } else {
        st.flags[3] = 1;
      }
      st.control[1] = slot + 1;
      st.control[2] = 1;
      st.control[kCtlSplit] = 0;  // cube_start is global again
      // the sum the reference normalises with is taken in the state dtype
      st.scalars[0] = (double)(T)(ds.s + ds.c);
      *a.ticket = 0u;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_finish_kernel(FinishArgs a) {
  finish_body<T>(a, blockIdx.x, gridDim.x);
}

// fp32 states: the per-cube terms in fp32 (the reference computes them in
// the state's dtype), every sum as a double-float on the FP32 pipe: per
// thread, over the CTA, and across CTAs in the last one.  The only FP64
// instructions are the two conversions of the cube's fp64 sums per cube.
__device__ __forceinline__ void f2_warp_sum3(F2& x, F2& y, F2& z) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const F2 x2 = f2_shfl_down(x, o), y2 = f2_shfl_down(y, o), z2 = f2_shfl_down(z, o);
    x = f2_add(x, x2);
    y = f2_add(y, y2);
    z = f2_add(z, z2);
  }
}

__device__ void finish_f32_body(const FinishArgs& a, unsigned bid, unsigned nblk) {
  __shared__ F2 sh[3][kBlock / 32];
  const tq_vegas_state& st = a.st;
  const float Vt = (float)a.V, V2t = (float)(a.V * a.V);
  const float beta = (float)a.beta;
  F2 res{0.f, 0.f}, s2{0.f, 0.f}, dsum{0.f, 0.f};
  const bool split = st.control[kCtlSplit] != 0;
  for (int64_t c = (int64_t)bid * blockDim.x + threadIdx.x; c < st.n_cubes;
       c += (int64_t)nblk * blockDim.x) {
    if (split) st.cube_start[c] += a.block_pre[c / kBlock];
    const int64_t nn = st.neval[c];
    const float cnt = (float)nn;  // the reference's JF / neval in the state dtype
    const float jT = __double2float_rn(st.jf[c]), j2T = __double2float_rn(st.jf2[c]);
    // vegas.py:294-303: ih = JF * V / n, sigma2 += |JF2 * V^2 / n - ih^2| / n
    const float inv = __frcp_rn(cnt);
    const float q = __fmul_rn(jT, inv);
    const float var = fabsf(__fmaf_rn(-q, q, __fmul_rn(j2T, inv)));
    res = f2_add(res, __fmul_rn(q, Vt));
    s2 = f2_add(s2, __fmul_rn(__fmul_rn(var, V2t), inv));
    // update_DH (vegas_stratification.py:72-86), reference operation order
    const float qd = div_rn(mul_rn(Vt, jT), cnt);
    float dt = sub_rn(div_rn(mul_rn(V2t, j2T), cnt), mul_rn(qd, qd));
    if (dt < 0.f) dt = 0.f;
    const float dh = (a.beta == 0.75) ? powf(dt, 0.75f) : powf(dt, beta);
    ((float*)st.dh)[c] = dh;
    dsum = f2_add(dsum, dh);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  f2_warp_sum3(res, s2, dsum);
  if (lane == 0) {
    sh[0][warp] = res;
    sh[1][warp] = s2;
    sh[2][warp] = dsum;
  }
  __syncthreads();
  F2* part = (F2*)a.partials;  // [blocks][3] double-floats in the Acc slots
  if (warp == 0) {
    const F2 zero{0.f, 0.f};
    res = lane < kBlock / 32 ? sh[0][lane] : zero;
    s2 = lane < kBlock / 32 ? sh[1][lane] : zero;
    dsum = lane < kBlock / 32 ? sh[2][lane] : zero;
    f2_warp_sum3(res, s2, dsum);
    if (lane == 0) {
      part[6 * bid] = res;
      part[6 * bid + 2] = s2;
      part[6 * bid + 4] = dsum;
    }
  }
  if (last_block_of(a.ticket, nblk) && warp == 0) {
    F2 r{0.f, 0.f}, q{0.f, 0.f}, ds{0.f, 0.f};
    for (unsigned i = lane; i < nblk; i += 32) {  // fixed assignment and tree: deterministic
      const float2 pr = __ldcg((const float2*)&part[6 * i]);
      const float2 pq = __ldcg((const float2*)&part[6 * i + 2]);
      const float2 pd = __ldcg((const float2*)&part[6 * i + 4]);
      r = f2_add(r, F2{pr.x, pr.y});
      q = f2_add(q, F2{pq.x, pq.y});
      ds = f2_add(ds, F2{pd.x, pd.y});
    }
    f2_warp_sum3(r, q, ds);
    if (lane == 0) {
      const int64_t slot = st.control[1];
      if (slot >= 0 && slot < st.n_stat_slots) {
        double* out = st.stats + 4 * slot;
        out[0] = f2_value(r);
        out[1] = f2_value(q);
        out[2] = (double)st.cube_start[st.n_cubes];
      } else {
        st.flags[3] = 1;
      }
      st.control[1] = slot + 1;
      st.control[2] = 1;
      st.control[kCtlSplit] = 0;  // cube_start is global again
      // the sum the reference normalises with is taken in the state dtype
      st.scalars[0] = (double)__fadd_rn(ds.hi, ds.lo);
      *a.ticket = 0u;
    }
  }
}

__global__ void __launch_bounds__(kBlock) vegas_finish_f32_kernel(FinishArgs a) {
  finish_f32_body(a, blockIdx.x, gridDim.x);
}

// --------------------------------------------------------- map update
// Block-wide sum (fp64), result in every thread.
__device__ double block_sum_all(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
  __syncthreads();
  return t;
}

constexpr int kSmallMap = 1024;  // intervals per dimension for the one-CTA-per-row path

// ------------------------------------------------ map update, large maps
// Maps of more than kSmallMap intervals per dimension (the reference's
// default N_increment // 10 intervals at large N): the update of
// vegas_map.py:114-260 as seven grid-wide passes over tiles of kMapTile
// intervals, grid (tiles, dimensions), so every SM takes part.  Stream order
// is the only grid-wide synchronisation.  Tile sums and tile prefixes are
// combined by the last CTA of a pass (ticket) in tile order, so results do
// not depend on CTA scheduling, and no CTA waits for another.
constexpr int kMapThreads = 256;
constexpr int kMapPer = 8;                       // consecutive intervals per thread
constexpr int kMapTile = kMapThreads * kMapPer;  // intervals per CTA
constexpr int kFillHalo = 16;  // 10 fill sweeps move values at most 10 intervals

inline int64_t map_tiles(int64_t B) { return (B + kMapTile - 1) / kMapTile; }

struct MapTiles {
  void* wf;       // [d][B]   T: averaged and filled weights (EQ 17)
  void* sw;       // [d][B]   T: smoothed weights (EQ 18-19)
  int32_t* mk;    // [d][B]   delta multiples of the fp64 cumulative sums
  int32_t* ind;   // [d][B+1] old interval index per new inner edge
  void* vv;       // [d][B+1] T: smoothed-weight sums per multiple
  void* newx;     // [d][B+1] T: new edges before the infinite-edge repair
  double* part;   // [d][nt]  tile sums
  double* pre;    // [d][nt]  exclusive tile prefixes
  double* row;    // [2][kMaxDim] row sums, deltas (T values)
  int* zero;      // some row of weights sums to zero: the map is reset
  size_t total;
};

static MapTiles map_tile_layout(const tq_vegas_state* st, void* base) {
  MapTiles m;
  const int64_t d = st->dim, B = st->n_bins, nt = map_tiles(B);
  const size_t ts = dtype_size(st->dtype);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  char* p = (char*)base;
  size_t off = 0;
  m.wf = p + off;   off += al(d * B * ts);
  m.sw = p + off;   off += al(d * B * ts);
  m.mk = (int32_t*)(p + off);  off += al(d * B * 4);
  m.ind = (int32_t*)(p + off); off += al(d * (B + 1) * 4);
  m.vv = p + off;   off += al(d * (B + 1) * ts);
  m.newx = p + off; off += al(d * (B + 1) * ts);
  m.part = (double*)(p + off); off += al(d * nt * 8);
  m.pre = (double*)(p + off);  off += al(d * nt * 8);
  m.row = (double*)(p + off);  off += al(2 * kMaxDim * 8);
  m.zero = (int*)(p + off);    off += 256;
  m.total = off;
  return m;
}

// Exclusive scan of one value per thread across the CTA (fixed order).
__device__ __forceinline__ double cta_exclusive_scan(double x, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double xi = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double v = __shfl_up_sync(0xffffffffu, xi, o);
    if (lane >= o) xi += v;
  }
  double ex = __shfl_up_sync(0xffffffffu, xi, 1);
  if (lane == 0) ex = 0.0;
  __syncthreads();
  if (lane == 31) sh[warp] = xi;
  __syncthreads();
  if (warp == 0) {
    double y = lane < nw ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double v = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += v;
    }
    double yx = __shfl_up_sync(0xffffffffu, y, 1);
    if (lane == 0) yx = 0.0;
    sh[lane] = yx;  // exclusive warp offsets
  }
  __syncthreads();
  const double r = sh[warp] + ex;
  __syncthreads();
  return r;
}

// Last CTA of a pass: per dimension, exclusive prefixes of the tile sums in
// tile order (one warp per dimension) and the row total.
__device__ void tile_prefixes(double* part, double* pre, double* total, int d, int64_t nt) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = warp; k < d; k += nw) {
    double carry = 0.0;
    for (int64_t c0 = 0; c0 < nt; c0 += 32) {
      const double v = c0 + lane < nt ? __ldcg(part + k * nt + c0 + lane) : 0.0;
      double xi = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, xi, o);
        if (lane >= o) xi += u;
      }
      double ex = __shfl_up_sync(0xffffffffu, xi, 1);
      if (lane == 0) ex = 0.0;
      if (pre && c0 + lane < nt) pre[k * nt + c0 + lane] = carry + ex;
      carry += __shfl_sync(0xffffffffu, xi, 31);
    }
    if (lane == 0) total[k] = carry;
  }
}

// Pass 1 (EQ 17, :118-145): averages, filling of empty intervals from their
// neighbours (10 sweeps on the tile plus a halo; once no empty interval is
// left a sweep changes nothing, so the reference's early exit needs no
// grid-wide test), tile sums; the last CTA forms the row sums and the
// zero-row test of :151-155.
template <typename T>
__global__ void __launch_bounds__(kMapThreads) map_fill_kernel(tq_vegas_state st, MapTiles m,
                                                                unsigned* ticket) {
  constexpr int E = kMapTile + 2 * kFillHalo;
  __shared__ T w_s[E], wt_s[E];
  __shared__ unsigned char z_s[E], zt_s[E];
  __shared__ double red[32];
  const int k = blockIdx.y;
  const int64_t B = st.n_bins, nt = gridDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * kMapTile, e0 = t0 - kFillHalo;
  int anyz = 0, rawz = 0;
  for (int i = threadIdx.x; i < E; i += blockDim.x) {
    const int64_t b = e0 + i;
    T wv = (T)0;
    unsigned char zv = 0;
    if (b >= 0 && b < B) {
      const int64_t c = st.counts[k * B + b];
      const T wi = (T)st.weights[k * B + b];
      zv = c == 0;
      wv = c == 0 ? wi : div_rn(wi, (T)c);
    }
    w_s[i] = wv;
    z_s[i] = zv;
    anyz |= zv;
    rawz |= zv && wv != (T)0;
  }
  // Empty intervals whose weights are zero (the only kind accumulation
  // produces): the 10 sweeps have a closed form.  Each sweep moves a fill
  // front one interval in from the nearest non-empty neighbour on each side,
  // the right one first, so an empty interval takes the value of the nearer
  // of its nearest non-empty neighbours within 10 intervals (the right one
  // on a tie) and stays empty beyond that.
  bool closed_form = false;
  if (__syncthreads_or(anyz)) closed_form = !__syncthreads_or(rawz);
  if (!closed_form && __syncthreads_or(anyz)) {
    for (int sweep = 0; sweep < 10; ++sweep) {
      for (int i = threadIdx.x; i < E; i += blockDim.x) {
        const bool right = e0 + i < B - 1 && i + 1 < E;
        wt_s[i] = (right && z_s[i]) ? w_s[i + 1] : w_s[i];
        zt_s[i] = right ? (z_s[i] && z_s[i + 1]) : z_s[i];
      }
      __syncthreads();
      for (int i = threadIdx.x; i < E; i += blockDim.x) {
        const bool left = e0 + i > 0 && i > 0;
        w_s[i] = (left && zt_s[i]) ? wt_s[i - 1] : wt_s[i];
        z_s[i] = left ? (zt_s[i] && zt_s[i - 1]) : zt_s[i];
      }
      __syncthreads();
    }
  }
  T* wf = (T*)m.wf + k * B;
  double acc = 0.0;
  for (int i = threadIdx.x; i < kMapTile; i += blockDim.x) {
    const int64_t b = t0 + i;
    if (b < B) {
      const int j = kFillHalo + i;
      T v = w_s[j];
      if (closed_form && z_s[j]) {
        int dr = 11, dl = 11;
        for (int q = 1; q <= 10 && b + q < B; ++q)
          if (!z_s[j + q]) {
            dr = q;
            break;
          }
        for (int q = 1; q <= 10 && b - q >= 0; ++q)
          if (!z_s[j - q]) {
            dl = q;
            break;
          }
        if (dr <= 10 || dl <= 10) v = dr <= dl ? w_s[j + dr] : w_s[j - dl];
      }
      wf[b] = v;
      acc += (double)v;
    }
  }
  acc = block_sum_all(acc, red);
  if (threadIdx.x == 0) m.part[k * nt + blockIdx.x] = acc;
  if (last_block_arrives(ticket)) {
    __threadfence();
    tile_prefixes(m.part, nullptr, m.row, st.dim, nt);
    __syncthreads();
    if (threadIdx.x == 0) {
      int z = 0;
      for (int kk = 0; kk < st.dim; ++kk) {
        const T s = (T)m.row[kk];
        m.row[kk] = (double)s;
        z |= s == (T)0;
      }
      *m.zero = z;
      *ticket = 0u;
    }
  }
}

// Pass 2 (EQ 18-19): smoothing and range compression; tile sums of the
// smoothed weights without the last interval (the fp64 cumulative sum of
// :210-213 runs over sw[:-1]); the last CTA forms the tile prefixes and
// delta = sum(sw) / B (:201).  smooth_only: _smooth_map alone (the result
// goes to sw, which then is the caller's buffer).
template <typename T>
__global__ void __launch_bounds__(kMapThreads) map_smooth_kernel(tq_vegas_state st, MapTiles m, double alpha,
                                                                  int smooth_only, unsigned* ticket) {
  __shared__ double red[32];
  if (*m.zero) {
    if (smooth_only && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(st.flags + 0, 1);
    return;
  }
  const int k = blockIdx.y;
  const int64_t B = st.n_bins, nt = gridDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * kMapTile;
  const T* r = (const T*)m.wf + k * B;
  T* sw = (T*)m.sw + k * B;
  const T sum = (T)m.row[k];
  double acc = 0.0;
  for (int i = threadIdx.x; i < kMapTile; i += blockDim.x) {
    const int64_t b = t0 + i;
    if (b >= B) break;
    T v;
    if (b == 0)
      v = add_rn(mul_rn((T)7, r[0]), r[1]);
    else if (b == B - 1)
      v = add_rn(r[B - 2], mul_rn((T)7, r[B - 1]));
    else
      v = add_rn(add_rn(r[b - 1], mul_rn((T)6, r[b])), r[b + 1]);
    v = div_rn(v, mul_rn((T)8, sum));
    if (v != (T)0) {
      const T t = div_rn(sub_rn(v, (T)1), log(v));
      v = alpha == 0.5 ? sqrt(t) : pow(t, (T)alpha);
    }
    sw[b] = v;
    if (b < B - 1) acc += (double)v;
  }
  if (smooth_only) return;
  acc = block_sum_all(acc, red);
  if (threadIdx.x == 0) m.part[k * nt + blockIdx.x] = acc;
  if (last_block_arrives(ticket)) {
    __threadfence();
    tile_prefixes(m.part, m.pre, m.row + kMaxDim, st.dim, nt);
    __syncthreads();
    if (threadIdx.x < st.dim) {
      const int kk = threadIdx.x;
      const double tot = m.row[kMaxDim + kk] + (double)__ldcg((const T*)m.sw + kk * B + B - 1);
      m.row[kMaxDim + kk] = (double)div_rn((T)tot, (T)B);
    }
    if (threadIdx.x == 0) *ticket = 0u;
  }
}

// Pass 3 (:210-213): fp64 cumulative sums of sw[:-1] (tile prefix + scan in
// the tile) divided by delta: the multiples; clears the per-multiple arrays.
template <typename T>
__global__ void __launch_bounds__(kMapThreads) map_multiples_kernel(tq_vegas_state st, MapTiles m) {
  __shared__ double red[32];
  if (*m.zero) return;
  const int k = blockIdx.y;
  const int64_t B = st.n_bins, nt = gridDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * kMapTile;
  const T* sw = (const T*)m.sw + k * B;
  const double delta = m.row[kMaxDim + k];
  const int64_t b0 = t0 + (int64_t)threadIdx.x * kMapPer;
  T v[kMapPer];
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < kMapPer; ++j) {
    v[j] = b0 + j < B - 1 ? sw[b0 + j] : (T)0;
    s += (double)v[j];
  }
  double cum = m.pre[k * nt + blockIdx.x] + cta_exclusive_scan(s, red);
  int32_t* mk = m.mk + k * B;
#pragma unroll
  for (int j = 0; j < kMapPer; ++j) {
    if (b0 + j < B - 1) {
      cum += (double)v[j];
      int64_t q;
      if constexpr (std::is_same<T, float>::value) {
        // floor(cum / delta) without an fp64 division: a float estimate,
        // then the exact test q * delta <= cum (q < 2^24 and delta a float,
        // so the product is exact in fp64)
        q = (int64_t)floorf(__fdiv_rn(__double2float_rn(cum), (float)delta));
        q = q < 0 ? 0 : (q > B + 1 ? B + 1 : q);
        if (q > 0 && (double)q * delta > cum) --q;
        else if ((double)(q + 1) * delta <= cum) ++q;
      } else {
        q = (int64_t)(cum / delta);
      }
      mk[b0 + j] = (int32_t)(q < 0 ? 0 : (q > B ? B : q));
    }
  }
  T* vv = (T*)m.vv + k * (B + 1);
  int32_t* ind = m.ind + k * (B + 1);
  for (int i = threadIdx.x; i < kMapTile; i += blockDim.x) {
    const int64_t e = t0 + i;
    if (e < B) {
      vv[e] = (T)0;
      ind[e] = 0;
    }
  }
  if (blockIdx.x == nt - 1 && threadIdx.x == 0) {
    vv[B] = (T)0;
    ind[B] = 0;
  }
}

// Pass 4 (:214-230) from the runs of equal multiples (mk nondecreasing):
// ind[e] = #{b : mk[b] <= e}, which is b for e in [mk[b-1], mk[b]), and
// vv[q] = the sequential sum (in T, as the reference's scatter-add) of sw
// over the run of multiple q.
constexpr int kRunHalo = 64;  // intervals past the tile staged for runs that cross its end

template <typename T>
__global__ void __launch_bounds__(kMapThreads) map_runs_kernel(tq_vegas_state st, MapTiles m) {
  __shared__ int32_t mk_s[kMapTile + kRunHalo + 1];  // [0] = mk[t0 - 1]
  __shared__ T sw_s[kMapTile + kRunHalo];
  if (*m.zero) return;
  const int k = blockIdx.y;
  const int64_t B = st.n_bins;
  const int64_t t0 = (int64_t)blockIdx.x * kMapTile;
  const int32_t* mk = m.mk + k * B;
  const T* sw = (const T*)m.sw + k * B;
  T* vv = (T*)m.vv + k * (B + 1);
  int32_t* ind = m.ind + k * (B + 1);
  // the multiples of intervals t0-1 .. t0+tile+halo-1 (those below B-1) and
  // their smoothed weights, so that runs are summed from shared memory
  const int64_t n_s = min((int64_t)(kMapTile + kRunHalo), B - 1 - t0);
  for (int i = threadIdx.x; i <= kMapTile + kRunHalo; i += blockDim.x) {
    const int64_t b = t0 - 1 + i;
    if (i == 0 || i - 1 < n_s) mk_s[i] = b >= 0 ? mk[b] : 0;
    if (i < n_s) sw_s[i] = sw[t0 + i];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kMapTile; i += blockDim.x) {
    const int64_t b = t0 + i;
    if (b >= B) break;
    const int64_t from = b == 0 ? 0 : mk_s[i];
    const int64_t to = b == B - 1 ? B + 1 : mk_s[i + 1];
    for (int64_t e = from; e < to; ++e) ind[e] = (int32_t)b;
    if (b < B - 1 && (b == 0 || mk_s[i + 1] != mk_s[i])) {
      const int32_t q = mk_s[i + 1];
      T a = (T)0;
      int64_t e = b;
      for (; e - t0 < n_s && mk_s[e - t0 + 1] == q; ++e) a = add_rn(a, sw_s[e - t0]);
      if (e - t0 >= n_s)  // a run longer than the staged halo
        for (; e < B - 1 && mk[e] == q; ++e) a = add_rn(a, sw[e]);
      vv[q] = a;
    }
  }
}

// Pass 5 (:233): tile sums of delta - vv[e] over e < B - 1; the last CTA
// forms the tile prefixes of the fp64 cumulative sum.
template <typename T>
__global__ void __launch_bounds__(kMapThreads) map_accu_sums_kernel(tq_vegas_state st, MapTiles m,
                                                                     unsigned* ticket) {
  __shared__ double red[32];
  if (*m.zero) return;
  const int k = blockIdx.y;
  const int64_t B = st.n_bins, nt = gridDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * kMapTile;
  const T delta = (T)m.row[kMaxDim + k];
  const T* vv = (const T*)m.vv + k * (B + 1);
  double acc = 0.0;
  for (int i = threadIdx.x; i < kMapTile; i += blockDim.x) {
    const int64_t e = t0 + i;
    if (e < B - 1) acc += (double)sub_rn(delta, vv[e]);
  }
  acc = block_sum_all(acc, red);
  if (threadIdx.x == 0) m.part[k * nt + blockIdx.x] = acc;
  if (last_block_arrives(ticket)) {
    __threadfence();
    tile_prefixes(m.part, m.pre, m.row, st.dim, nt);  // row sums are no longer needed
    __syncthreads();
    if (threadIdx.x == 0) *ticket = 0u;
  }
}

// Pass 6 (:233-238, EQ 22): d_accu (fp64 cumulative sum rounded to T per
// element, as torch's CPU cumsum) and the new inner edges.
template <typename T>
__global__ void __launch_bounds__(kMapThreads) map_edges_kernel(tq_vegas_state st, MapTiles m) {
  __shared__ double red[32];
  if (*m.zero) return;
  const int k = blockIdx.y;
  const int64_t B = st.n_bins, nt = gridDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * kMapTile;
  const T delta = (T)m.row[kMaxDim + k];
  const T* vv = (const T*)m.vv + k * (B + 1);
  const T* sw = (const T*)m.sw + k * B;
  const int32_t* ind = m.ind + k * (B + 1);
  const T* xe = (const T*)st.x_edges + k * (B + 1);
  const T* dxe = (const T*)st.dx_edges + k * B;
  T* nx = (T*)m.newx + k * (B + 1);
  const int64_t e0 = t0 + (int64_t)threadIdx.x * kMapPer;
  double x[kMapPer];
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < kMapPer; ++j) {
    x[j] = e0 + j < B - 1 ? (double)sub_rn(delta, vv[e0 + j]) : 0.0;
    s += x[j];
  }
  double cum = m.pre[k * nt + blockIdx.x] + cta_exclusive_scan(s, red);
#pragma unroll
  for (int j = 0; j < kMapPer; ++j) {
    const int64_t e = e0 + j;
    if (e < B - 1) {
      cum += x[j];
      const T da = (T)cum;
      int64_t ii = ind[e];
      ii = ii < 0 ? 0 : (ii > B - 1 ? B - 1 : ii);
      nx[e + 1] = add_rn(xe[ii], mul_rn(div_rn(da, sw[ii]), dxe[ii]));
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    nx[0] = xe[0];
    nx[B] = xe[B];
  }
}

// Pass 7 (:239-262): infinite edges replaced by the mean of their two
// (unrepaired) neighbours, new edges and widths stored, weights and counts
// reset; or, for a map that cannot be updated, only the reset.
template <typename T>
__global__ void __launch_bounds__(kMapThreads) map_commit_kernel(tq_vegas_state st, MapTiles m) {
  const int k = blockIdx.y;
  const int64_t B = st.n_bins;
  const int64_t t0 = (int64_t)blockIdx.x * kMapTile;
  const bool reset_only = *m.zero != 0;
  if (reset_only && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(st.flags + 0, 1);
  const T* nx = (const T*)m.newx + k * (B + 1);
  T* xe = (T*)st.x_edges + k * (B + 1);
  T* dxe = (T*)st.dx_edges + k * B;
  auto fixed = [&](int64_t e, bool count) -> T {
    T v = nx[e];
    if (!isfinite((double)v)) {
      if (count) atomicAdd(st.flags + 1, 1);
      if (e > 0 && e < B) v = mul_rn((T)0.5, add_rn(nx[e - 1], nx[e + 1]));
      if (count && !isfinite((double)v)) atomicAdd(st.flags + 2, 1);
    }
    return v;
  };
  for (int i = threadIdx.x; i < kMapTile; i += blockDim.x) {
    const int64_t b = t0 + i;
    if (b >= B) break;
    if (!reset_only) {
      const T lo = fixed(b, true);
      const T hi = fixed(b + 1, b == B - 1);
      xe[b] = lo;
      if (b == B - 1) xe[B] = hi;
      dxe[b] = sub_rn(hi, lo);
    }
    st.weights[k * B + b] = 0.0;
    st.counts[k * B + b] = 0;
  }
}

// ------------------------------------------------ map update, small maps
// Maps of at most kSmallMap intervals per dimension: one CTA per dimension
// runs the whole update of vegas_map.py:114-260 for its row in shared
// memory, the cumulative sums as block scans.  The map-wide "some row of
// weights sums to zero" test (:151-155) is made by every CTA over the whole
// map: the weights are sums of squares, so a row of averaged (and filled)
// weights sums to zero exactly when each of its averages is zero.  Since
// every CTA reads every row, the weights and counts are cleared by the last
// CTA to finish (ticket), not by each CTA for its own row.
constexpr int kRowThreads = 256;
constexpr int kRowPer = kSmallMap / kRowThreads;  // consecutive intervals per thread in the scans

inline size_t map_row_smem(int64_t B, size_t ts) {
  return (((7 * B + 3) * ts + (2 * B + 1) * 4 + 2 * B) + 15) & ~size_t(15);
}

// The last CTA to arrive resets the weights and counts of the whole map
// (_reset_weight).  Every CTA read the whole map's weights and counts; the
// fenced ticket (last_block_of) orders those reads before the reset.
__device__ void clear_map_by_last(const tq_vegas_state& st, unsigned* ticket, unsigned nrows) {
  if (last_block_of(ticket, nrows)) {
    const int64_t n = (int64_t)st.dim * st.n_bins;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      st.weights[i] = 0.0;
      st.counts[i] = 0;
    }
    if (threadIdx.x == 0) *ticket = 0u;
  }
}

template <typename T>
__device__ void map_rows_body(const tq_vegas_state& st, double alpha, void* smooth_out, unsigned* ticket,
                              int k, unsigned nrows) {
  extern __shared__ __align__(16) unsigned char row_smem[];
  __shared__ double red[32];
  __shared__ int rownz[kMaxDim];
  const int d = st.dim;
  const int B = (int)st.n_bins;
  T* w = (T*)row_smem;                                 // [B] averaged, filled weights
  T* wt = w + B;                                       // [B]
  T* sw = wt + B;                                      // [B] smoothed weights
  T* vv = sw + B;                                      // [B+1] sums per delta multiple
  T* nx = vv + (B + 1);                                // [B+1] new edges
  int32_t* mk = (int32_t*)(nx + (B + 1));              // [B] delta multiples
  int32_t* ind = mk + B;                               // [B+1] old interval per new edge
  unsigned char* z = (unsigned char*)(ind + (B + 1));  // [B] empty intervals
  unsigned char* zt = z + B;                           // [B]
  // zero-row test over the whole map
  if (threadIdx.x < d) rownz[threadIdx.x] = 0;
  __syncthreads();
  for (int kk = 0; kk < d; ++kk) {
    int nz = 0;
    for (int b = threadIdx.x; b < B; b += blockDim.x) {
      const int64_t c = st.counts[(int64_t)kk * B + b];
      const T wi = (T)st.weights[(int64_t)kk * B + b];
      nz |= (c == 0 ? wi : div_rn(wi, (T)c)) != (T)0;
    }
    if (nz) rownz[kk] = 1;
  }
  __syncthreads();
  int zero_row = 0;
  for (int kk = 0; kk < d; ++kk) zero_row |= !rownz[kk];
  if (zero_row) {  // the map cannot be updated (:187-196): only the reset
    if (k == 0 && threadIdx.x == 0) atomicAdd(st.flags + 0, 1);
    if (!smooth_out) clear_map_by_last(st, ticket, nrows);
    return;
  }
  // EQ 17 and the filling of empty intervals (:118-145).  A sweep over a row
  // without empty intervals changes nothing, so stopping per row gives the
  // reference's map-wide stopping rule.
  int anyz = 0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const int64_t c = st.counts[(int64_t)k * B + b];
    const T wi = (T)st.weights[(int64_t)k * B + b];
    z[b] = c == 0;
    anyz |= c == 0;
    w[b] = c == 0 ? wi : div_rn(wi, (T)c);
  }
  if (__syncthreads_or(anyz)) {
    for (int sweep = 0; sweep < 10; ++sweep) {
      for (int b = threadIdx.x; b < B; b += blockDim.x) {
        wt[b] = (b < B - 1 && z[b]) ? w[b + 1] : w[b];
        zt[b] = (b < B - 1) ? (z[b] && z[b + 1]) : z[b];
      }
      __syncthreads();
      int left = 0;
      for (int b = threadIdx.x; b < B; b += blockDim.x) {
        w[b] = (b > 0 && zt[b]) ? wt[b - 1] : wt[b];
        z[b] = (b > 0) ? (zt[b] && zt[b - 1]) : zt[b];
        left |= z[b];
      }
      if (!__syncthreads_or(left)) break;
    }
  }
  double acc = 0.0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) acc += (double)w[b];
  const T sum = (T)block_sum_all(acc, red);  // :151
  // EQ 18-19
  acc = 0.0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    T v;
    if (b == 0)
      v = add_rn(mul_rn((T)7, w[0]), w[1]);
    else if (b == B - 1)
      v = add_rn(w[B - 2], mul_rn((T)7, w[B - 1]));
    else
      v = add_rn(add_rn(w[b - 1], mul_rn((T)6, w[b])), w[b + 1]);
    v = div_rn(v, mul_rn((T)8, sum));
    if (v != (T)0) {
      const T t = div_rn(sub_rn(v, (T)1), log(v));
      v = alpha == 0.5 ? sqrt(t) : pow(t, (T)alpha);
    }
    sw[b] = v;
    acc += (double)v;
    if (smooth_out) ((T*)smooth_out)[(int64_t)k * B + b] = v;
  }
  if (smooth_out) return;  // _smooth_map only: the map and its weights stay
  const T delta = div_rn((T)block_sum_all(acc, red), (T)B);  // :201 (the barrier publishes sw)
  // :210-213: fp64 cumulative sums of sw[:-1] divided by delta
  const int b0 = threadIdx.x * kRowPer;
  double x[kRowPer];
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < kRowPer; ++j) {
    x[j] = b0 + j < B - 1 ? (double)sw[b0 + j] : 0.0;
    s += x[j];
  }
  double cum = cta_exclusive_scan(s, red);
#pragma unroll
  for (int j = 0; j < kRowPer; ++j) {
    if (b0 + j < B - 1) {
      cum += x[j];
      const int64_t q = (int64_t)(cum / (double)delta);
      mk[b0 + j] = (int32_t)(q < 0 ? 0 : (q > B ? B : q));
    }
  }
  for (int e = threadIdx.x; e <= B; e += blockDim.x) {
    vv[e] = (T)0;
    ind[e] = 0;
  }
  __syncthreads();
  // :214-230 from the runs of equal multiples: ind[e] = #{b : mk[b] <= e},
  // vv[q] = the sequential sum of sw over the run of multiple q
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const int from = b == 0 ? 0 : mk[b - 1];
    const int to = b == B - 1 ? B + 1 : mk[b];
    for (int e = from; e < to; ++e) ind[e] = b;
    if (b < B - 1 && (b == 0 || mk[b] != mk[b - 1])) {
      const int q = mk[b];
      T a = (T)0;
      for (int e = b; e < B - 1 && mk[e] == q; ++e) a = add_rn(a, sw[e]);
      vv[q] = a;
    }
  }
  __syncthreads();
  // :233 d_accu (fp64 cumulative sum rounded to T per element) and EQ 22
  const T* xe = (const T*)st.x_edges + (int64_t)k * (B + 1);
  const T* dxe = (const T*)st.dx_edges + (int64_t)k * B;
  s = 0.0;
#pragma unroll
  for (int j = 0; j < kRowPer; ++j) {
    x[j] = b0 + j < B - 1 ? (double)sub_rn(delta, vv[b0 + j]) : 0.0;
    s += x[j];
  }
  cum = cta_exclusive_scan(s, red);
#pragma unroll
  for (int j = 0; j < kRowPer; ++j) {
    const int e = b0 + j;
    if (e < B - 1) {
      cum += x[j];
      int ii = ind[e];
      ii = ii < 0 ? 0 : (ii > B - 1 ? B - 1 : ii);
      nx[e + 1] = add_rn(xe[ii], mul_rn(div_rn((T)cum, sw[ii]), dxe[ii]));
    }
  }
  if (threadIdx.x == 0) {
    nx[0] = xe[0];
    nx[B] = xe[B];
  }
  __syncthreads();
  // :239-257: infinite edges replaced by the mean of their neighbours (rare)
  int bad = 0;
  for (int e = threadIdx.x; e <= B; e += blockDim.x) bad |= !isfinite((double)nx[e]);
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) {
      atomicAdd(st.flags + 1, 1);
      for (int e = 1; e < B; ++e) vv[e] = mul_rn((T)0.5, add_rn(nx[e - 1], nx[e + 1]));
      for (int e = 1; e < B; ++e)
        if (!isfinite((double)nx[e])) nx[e] = vv[e];
      for (int e = 0; e <= B; ++e)
        if (!isfinite((double)nx[e])) {
          atomicAdd(st.flags + 2, 1);
          break;
        }
    }
    __syncthreads();
  }
  T* xo = (T*)st.x_edges + (int64_t)k * (B + 1);
  T* dxo = (T*)st.dx_edges + (int64_t)k * B;
  for (int e = threadIdx.x; e <= B; e += blockDim.x) xo[e] = nx[e];
  for (int b = threadIdx.x; b < B; b += blockDim.x) dxo[b] = sub_rn(nx[b + 1], nx[b]);  // :259
  clear_map_by_last(st, ticket, nrows);
}

template <typename T>
__global__ void __launch_bounds__(kRowThreads) vegas_map_rows_kernel(tq_vegas_state st, double alpha,
                                                                      void* smooth_out, unsigned* ticket) {
  map_rows_body<T>(st, alpha, smooth_out, ticket, blockIdx.x, gridDim.x);
}

// fp32 maps: the same update with every fp64 sum and scan of the generic
// kernel as a double-float on the FP32 pipe (the reference's fp64
// cumulative sums of fp32 values are exact in both forms whenever they are
// exact in fp64).  The delta multiple of a cumulative sum C = hi + lo is the
// largest k with k * delta <= C, decided from the exact residual (k * delta
// as a TwoProduct): multiples agree with the fp64 truncation except where
// C / delta lies within about 2^-46 of an integer without being one.
__device__ F2 f2_block_sum_all(F2 v, F2* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = f2_add(v, f2_shfl_down(v, o));
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {  // the warp partials in a fixed tree
    F2 t = lane < nw ? sh[lane] : F2{0.f, 0.f};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = f2_add(t, f2_shfl_down(t, o));
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

__device__ F2 f2_cta_exclusive_scan(F2 x, F2* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  F2 xi = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const F2 v = f2_shfl_up(xi, o);
    if (lane >= o) xi = f2_add(v, xi);
  }
  F2 ex = f2_shfl_up(xi, 1);
  if (lane == 0) ex = F2{0.f, 0.f};
  __syncthreads();
  if (lane == 31) sh[warp] = xi;
  __syncthreads();
  if (warp == 0) {
    F2 y = lane < nw ? sh[lane] : F2{0.f, 0.f};
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const F2 v = f2_shfl_up(y, o);
      if (lane >= o) y = f2_add(v, y);
    }
    F2 yx = f2_shfl_up(y, 1);
    if (lane == 0) yx = F2{0.f, 0.f};
    sh[lane] = yx;
  }
  __syncthreads();
  const F2 r = f2_add(sh[warp], ex);
  __syncthreads();
  return r;
}

// C = c.hi + c.lo >= k * delta, exactly up to the last two roundings.
__device__ __forceinline__ bool f2_at_least(F2 c, int k, float delta) {
  const float kf = (float)k;
  const float ph = __fmul_rn(kf, delta);
  const float pl = __fmaf_rn(kf, delta, -ph);  // k * delta = ph + pl exactly
  const float r = __fsub_rn(__fadd_rn(__fsub_rn(c.hi, ph), c.lo), pl);
  return r >= 0.f;
}

__device__ void map_rows_f32_body(const tq_vegas_state& st, double alpha, void* smooth_out, unsigned* ticket,
                                  int k, unsigned nrows) {
  using T = float;
  extern __shared__ __align__(16) unsigned char row_smem[];
  __shared__ F2 red[33];
  __shared__ int rownz[kMaxDim];
  const int d = st.dim;
  const int B = (int)st.n_bins;
  T* w = (T*)row_smem;
  T* wt = w + B;
  T* sw = wt + B;
  T* vv = sw + B;
  T* nx = vv + (B + 1);
  T* xe = nx + (B + 1);  // [B+1] old edges
  T* dxe = xe + (B + 1);  // [B] old widths
  int32_t* mk = (int32_t*)(dxe + B);
  int32_t* ind = mk + B;
  unsigned char* z = (unsigned char*)(ind + (B + 1));
  unsigned char* zt = z + B;
  // one pass over global memory: the zero-row test over every row (all
  // elements of the map at once), this row's averages and empty intervals,
  // and this row's edges
  if (threadIdx.x < d) rownz[threadIdx.x] = 0;
  __syncthreads();
  const T* xe_g = (const T*)st.x_edges + (int64_t)k * (B + 1);
  const T* dxe_g = (const T*)st.dx_edges + (int64_t)k * B;
  if (!smooth_out) {
    for (int e = threadIdx.x; e <= B; e += blockDim.x) xe[e] = xe_g[e];
    for (int b = threadIdx.x; b < B; b += blockDim.x) dxe[b] = dxe_g[b];
  }
  int anyz = 0;
  for (int i = threadIdx.x; i < d * B; i += blockDim.x) {
    const int64_t c = st.counts[i];
    const T wi = (T)st.weights[i];
    const T av = c == 0 ? wi : div_rn(wi, (T)c);
    const int kk = i / B, b = i - kk * B;
    if (av != (T)0 && !rownz[kk]) rownz[kk] = 1;
    if (kk == k) {
      z[b] = c == 0;
      anyz |= c == 0;
      w[b] = av;
    }
  }
  __syncthreads();
  int zero_row = 0;
  for (int kk = 0; kk < d; ++kk) zero_row |= !rownz[kk];
  if (zero_row) {
    if (k == 0 && threadIdx.x == 0) atomicAdd(st.flags + 0, 1);
    if (!smooth_out) clear_map_by_last(st, ticket, nrows);
    return;
  }
  if (__syncthreads_or(anyz)) {
    for (int sweep = 0; sweep < 10; ++sweep) {
      for (int b = threadIdx.x; b < B; b += blockDim.x) {
        wt[b] = (b < B - 1 && z[b]) ? w[b + 1] : w[b];
        zt[b] = (b < B - 1) ? (z[b] && z[b + 1]) : z[b];
      }
      __syncthreads();
      int left = 0;
      for (int b = threadIdx.x; b < B; b += blockDim.x) {
        w[b] = (b > 0 && zt[b]) ? wt[b - 1] : wt[b];
        z[b] = (b > 0) ? (zt[b] && zt[b - 1]) : zt[b];
        left |= z[b];
      }
      if (!__syncthreads_or(left)) break;
    }
  }
  F2 acc{0.f, 0.f};
  for (int b = threadIdx.x; b < B; b += blockDim.x) acc = f2_add(acc, w[b]);
  const T sum = f2_round(f2_block_sum_all(acc, red));  // :151
  acc = F2{0.f, 0.f};
  for (int b = threadIdx.x; b < B; b += blockDim.x) {  // EQ 18-19
    T v;
    if (b == 0)
      v = add_rn(mul_rn((T)7, w[0]), w[1]);
    else if (b == B - 1)
      v = add_rn(w[B - 2], mul_rn((T)7, w[B - 1]));
    else
      v = add_rn(add_rn(w[b - 1], mul_rn((T)6, w[b])), w[b + 1]);
    v = div_rn(v, mul_rn((T)8, sum));
    if (v != (T)0) {
      const T t = div_rn(sub_rn(v, (T)1), logf(v));
      v = alpha == 0.5 ? sqrtf(t) : powf(t, (T)alpha);
    }
    sw[b] = v;
    acc = f2_add(acc, v);
    if (smooth_out) ((T*)smooth_out)[(int64_t)k * B + b] = v;
  }
  if (smooth_out) return;
  const T delta = div_rn(f2_round(f2_block_sum_all(acc, red)), (T)B);  // :201
  // :210-213: cumulative sums of sw[:-1] (each thread a contiguous chunk,
  // one interval for maps up to 257 intervals), their delta multiples
  const int per = (B - 1 + (int)blockDim.x - 1) / (int)blockDim.x;
  const int b0 = threadIdx.x * per, b1 = min(B - 1, b0 + per);
  F2 s{0.f, 0.f};
  for (int b = b0; b < b1; ++b) s = f2_add(s, sw[b]);
  F2 cum = f2_cta_exclusive_scan(s, red);
  for (int b = b0; b < b1; ++b) {
    cum = f2_add(cum, sw[b]);
    int q = (int)floorf(__fdiv_rn(cum.hi, delta));
    q = q < 0 ? 0 : (q > B + 1 ? B + 1 : q);
    if (q > 0 && !f2_at_least(cum, q, delta)) --q;
    else if (f2_at_least(cum, q + 1, delta)) ++q;
    mk[b] = q > B ? B : q;
  }
  for (int e = threadIdx.x; e <= B; e += blockDim.x) {
    vv[e] = (T)0;
    ind[e] = 0;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < B; b += blockDim.x) {  // :214-230
    const int from = b == 0 ? 0 : mk[b - 1];
    const int to = b == B - 1 ? B + 1 : mk[b];
    for (int e = from; e < to; ++e) ind[e] = b;
    if (b < B - 1 && (b == 0 || mk[b] != mk[b - 1])) {
      const int q = mk[b];
      T a = (T)0;
      for (int e = b; e < B - 1 && mk[e] == q; ++e) a = add_rn(a, sw[e]);
      vv[q] = a;
    }
  }
  __syncthreads();
  // :233 d_accu and EQ 22
  s = F2{0.f, 0.f};
  for (int e = b0; e < b1; ++e) s = f2_add(s, sub_rn(delta, vv[e]));
  cum = f2_cta_exclusive_scan(s, red);
  for (int e = b0; e < b1; ++e) {
    cum = f2_add(cum, sub_rn(delta, vv[e]));
    int ii = ind[e];
    ii = ii < 0 ? 0 : (ii > B - 1 ? B - 1 : ii);
    nx[e + 1] = add_rn(xe[ii], mul_rn(div_rn(f2_round(cum), sw[ii]), dxe[ii]));
  }
  if (threadIdx.x == 0) {
    nx[0] = xe[0];
    nx[B] = xe[B];
  }
  __syncthreads();
  int bad = 0;
  for (int e = threadIdx.x; e <= B; e += blockDim.x) bad |= !isfinite(nx[e]);
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) {
      atomicAdd(st.flags + 1, 1);
      for (int e = 1; e < B; ++e) vv[e] = mul_rn((T)0.5, add_rn(nx[e - 1], nx[e + 1]));
      for (int e = 1; e < B; ++e)
        if (!isfinite(nx[e])) nx[e] = vv[e];
      for (int e = 0; e <= B; ++e)
        if (!isfinite(nx[e])) {
          atomicAdd(st.flags + 2, 1);
          break;
        }
    }
    __syncthreads();
  }
  T* xo = (T*)st.x_edges + (int64_t)k * (B + 1);
  T* dxo = (T*)st.dx_edges + (int64_t)k * B;
  for (int e = threadIdx.x; e <= B; e += blockDim.x) xo[e] = nx[e];
  for (int b = threadIdx.x; b < B; b += blockDim.x) dxo[b] = sub_rn(nx[b + 1], nx[b]);  // :259
  clear_map_by_last(st, ticket, nrows);
}

__global__ void __launch_bounds__(kRowThreads) vegas_map_rows_f32_kernel(tq_vegas_state st, double alpha,
                                                                          void* smooth_out, unsigned* ticket) {
  map_rows_f32_body(st, alpha, smooth_out, ticket, blockIdx.x, gridDim.x);
}

// finish_iteration and update_map in one launch (maps of at most kSmallMap
// intervals): CTAs 0..d-1 update the map rows, the others end the
// iteration.  The two read and write disjoint parts of the state, so they
// run side by side; each role counts its own CTAs on its own ticket.
template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_finish_map_kernel(FinishArgs a, double alpha,
                                                                  unsigned* map_ticket) {
  const unsigned d = (unsigned)a.st.dim;
  if (blockIdx.x < d) {
    if constexpr (std::is_same<T, float>::value)
      map_rows_f32_body(a.st, alpha, nullptr, map_ticket, blockIdx.x, d);
    else
      map_rows_body<T>(a.st, alpha, nullptr, map_ticket, blockIdx.x, d);
  } else {
    if constexpr (std::is_same<T, float>::value)
      finish_f32_body(a, blockIdx.x - d, gridDim.x - d);
    else
      finish_body<T>(a, blockIdx.x - d, gridDim.x - d);
  }
}

// ----------------------------------------------------------- init
template <typename T>
__global__ void vegas_init_kernel(tq_vegas_state st) {
  const int d = st.dim;
  const int64_t B = st.n_bins;
  const T step = div_rn((T)1, (T)B);  // linspace(0, 1, B+1) step
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < d * (B + 1);
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i % (B + 1);
    ((T*)st.x_edges)[i] = linspace_node<T>((T)0, (T)1, step, B + 1, b);
  }
  const T inv = div_rn((T)1, (T)B);  // ones / N_intervals (vegas_map.py:34-37)
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < d * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    ((T*)st.dx_edges)[i] = inv;
    st.weights[i] = 0.0;
    st.counts[i] = 0;
  }
  // dh = ones * 1.0 / N_cubes (vegas_stratification.py:40)
  const T dh0 = div_rn((T)1, (T)st.n_cubes);
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < st.n_cubes;
       c += (int64_t)gridDim.x * blockDim.x) {
    ((T*)st.dh)[c] = dh0;
    st.jf[c] = 0.0;
    st.jf2[c] = 0.0;
    st.neval[c] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x < 4) {
    st.flags[threadIdx.x] = 0;
    st.scalars[threadIdx.x] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st.control[1] = 0;
    st.control[2] = 0;
    st.control[kCtlSplit] = 0;
  }
}

__global__ void vegas_set_control_kernel(int64_t* control, int mask, int64_t nevals, int64_t slot,
                                         int64_t normalize, uint64_t seed, uint64_t sid) {
  if (mask & TQ_VC_NEVALS) control[0] = nevals;
  if (mask & TQ_VC_SLOT) control[1] = slot;
  if (mask & TQ_VC_NORMALIZE) control[2] = normalize;
  if (mask & TQ_VC_SEED) control[3] = (int64_t)seed;
  if (mask & TQ_VC_STREAM) control[4] = (int64_t)sid;
}

// ------------------------------------------------ materialised kernels
template <typename T>
__global__ void __launch_bounds__(kTile) vegas_strat_points_kernel(tq_vegas_state st, const T* u,
                                                                   int64_t M, T* y) {
  const int d = st.dim;
  const int64_t ns = st.n_strat;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M;
       j += (int64_t)gridDim.x * blockDim.x) {
    // cube of point j: binary search in cube_start
    int64_t l = 0, h = st.n_cubes;
    while (h - l > 1) {
      const int64_t m = (l + h) >> 1;
      if (st.cube_start[m] <= j) l = m;
      else h = m;
    }
    int64_t cc = l;
    const T nsf = (T)ns;
    for (int k = 0; k < d; ++k) {
      const int64_t q = cc / ns;
      y[j * d + k] = strat_y<T>((int)(cc - q * ns), u[j * d + k], nsf);
      cc = q;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kTile) vegas_map_points_kernel(tq_vegas_state st, const T* y,
                                                                 int64_t M, T* x, T* jac) {
  const int d = st.dim;
  const int B = (int)st.n_bins;
  const T Bf = (T)B;
  const T* xe = (const T*)st.x_edges;
  const T* dxe = (const T*)st.dx_edges;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M;
       j += (int64_t)gridDim.x * blockDim.x) {
    T jc = (T)1;
    for (int k = 0; k < d; ++k) {
      T xv, jf;
      map_coord<T>(xe + k * (B + 1), dxe + k * B, B, Bf, y[j * d + k], xv, jf);
      x[j * d + k] = xv;
      jc = mul_rn(jc, jf);
    }
    jac[j] = jc;
  }
}

template <typename T>
__global__ void __launch_bounds__(kTile) vegas_accumulate_kernel(tq_vegas_state st, const T* y,
                                                                 const T* vals, int64_t M,
                                                                 int acc_map, int stratified) {
  const int d = st.dim;
  const int64_t B = st.n_bins;
  const T Bf = (T)B;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M;
       j += (int64_t)gridDim.x * blockDim.x) {
    const T v = vals[j];
    const double v2 = (double)v * (double)v;
    if (acc_map) {
      for (int k = 0; k < d; ++k) {
        int id = (int)floor(mul_rn(y[j * d + k], Bf));
        id = id < 0 ? 0 : (id >= (int)B ? (int)B - 1 : id);
        atomicAdd(st.weights + k * B + id, (double)v);
        atomicAdd((unsigned long long*)(st.counts + k * B + id), 1ull);
      }
    }
    if (stratified) {
      int64_t l = 0, h = st.n_cubes;
      while (h - l > 1) {
        const int64_t m = (l + h) >> 1;
        if (st.cube_start[m] <= j) l = m;
        else h = m;
      }
      atomicAdd(st.jf + l, (double)v);
      atomicAdd(st.jf2 + l, v2);
    }
  }
}

}  // namespace tq

using namespace tq;

// ----------------------------------------------------------------- C ABI
static int check_state(const tq_vegas_state* st) {
  if (!st) return TQ_ERR_ARG;
  if (!valid_dtype(st->dtype)) return TQ_ERR_DTYPE;
  if (st->dim < 1 || st->dim > kMaxDim) return TQ_ERR_DIM;
  if (st->n_bins < 2 || st->n_strat < 1 || st->n_cubes < 1 || st->n_bins > (int64_t(1) << 30))
    return TQ_ERR_ARG;
  int64_t nc = 1;
  for (int k = 0; k < st->dim; ++k) {
    if (nc > (int64_t(1) << 40) / st->n_strat) return TQ_ERR_TOO_LARGE;
    nc *= st->n_strat;
  }
  if (nc != st->n_cubes) return TQ_ERR_ARG;
  if (!st->x_edges || !st->dx_edges || !st->weights || !st->counts || !st->dh || !st->jf ||
      !st->jf2 || !st->neval || !st->cube_start || !st->rng_offset || !st->stats || !st->flags ||
      !st->scalars || !st->domain || !st->control || st->n_stat_slots < 1)
    return TQ_ERR_ARG;
  return TQ_OK;
}

static int64_t nh_blocks(const tq_vegas_state* st) { return (st->n_cubes + kBlock - 1) / kBlock; }
static int64_t finish_blocks(const tq_vegas_state* st) {
  const int64_t need = (st->n_cubes + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)sm_count() * 2;
  return need < cap ? need : cap;
}
static size_t map_scratch_bytes(const tq_vegas_state* st) {
  if (st->n_bins > kSmallMap) return map_tile_layout(st, nullptr).total;
  return 256;
}

// Workspace: [0,256) tickets; then nh block totals, finish partials and the
// map-update scratch, each 256-byte aligned.
struct VegasWs {
  unsigned* t_sample;
  unsigned* t_nh;
  unsigned* t_finish;
  unsigned* t_map;
  int64_t* block_tot;
  Acc* partials;
  double* map_scratch;
  size_t total;
};
static VegasWs vegas_ws(const tq_vegas_state* st, void* base) {
  VegasWs w;
  char* p = (char*)base;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  w.t_sample = (unsigned*)(p + 0);
  w.t_nh = (unsigned*)(p + 16);
  w.t_finish = (unsigned*)(p + 32);
  w.t_map = (unsigned*)(p + 64);  // three tickets, 16 bytes apart
  size_t off = 256;
  w.block_tot = (int64_t*)(p + off);
  off += al(sizeof(int64_t) * (size_t)nh_blocks(st));
  w.partials = (Acc*)(p + off);
  off += al(sizeof(Acc) * 3 * (size_t)finish_blocks(st));
  w.map_scratch = (double*)(p + off);
  off += al(map_scratch_bytes(st));
  w.total = off;
  return w;
}

extern "C" size_t tq_vegas_workspace_size(const tq_vegas_state* st) {
  if (check_state(st) != TQ_OK) return 0;
  return vegas_ws(st, nullptr).total;
}

#define TQ_VEGAS_WS()                                              \
  int rc = check_state(st);                                        \
  if (rc != TQ_OK) return rc;                                      \
  if (!workspace) return TQ_ERR_ARG;                               \
  VegasWs ws = vegas_ws(st, workspace);                            \
  if (workspace_bytes < ws.total) return TQ_ERR_WORKSPACE;         \
  cudaStream_t s = (cudaStream_t)stream;

extern "C" int tq_vegas_init(const tq_vegas_state* st, void* stream) {
  const int rc = check_state(st);
  if (rc != TQ_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t work = st->n_cubes > st->dim * (st->n_bins + 1) ? st->n_cubes : st->dim * (st->n_bins + 1);
  int64_t g = (work + kBlock - 1) / kBlock;
  if (g > (int64_t)sm_count() * 8) g = (int64_t)sm_count() * 8;
  if (st->dtype == TQ_F64)
    vegas_init_kernel<double><<<(unsigned)g, kBlock, 0, s>>>(*st);
  else
    vegas_init_kernel<float><<<(unsigned)g, kBlock, 0, s>>>(*st);
  return launch_status();
}

static int launch_sample(const tq_vegas_state* st, int family, const double* params,
                         int64_t n_samples, int use_map, int64_t max_points, bool warm,
                         unsigned* ticket, const int64_t* block_pre, cudaStream_t s) {
  SampleArgs a;
  a.st = *st;
  a.family = family;
  a.params = params;
  a.n_samples = n_samples;
  a.use_map = use_map;
  a.ticket = ticket;
  a.block_pre = block_pre;
  a.small_cubes = st->n_cubes < (int64_t(1) << 32) && st->n_strat < (int64_t(1) << 31);
  a.ns_div = make_fastdiv((uint32_t)(a.small_cubes ? st->n_strat : 1));
  const size_t tsize = dtype_size(st->dtype);
  const size_t limit = 96 * 1024;
  a.hist_smem = sample_smem_bytes(st->dim, st->n_bins, tsize, true, false) <= limit / 2 &&
                st->dim * st->n_bins < (int64_t(1) << 30);
  a.edges_smem = sample_smem_bytes(st->dim, st->n_bins, tsize, a.hist_smem, true) <= limit;
  const size_t smem = sample_smem_bytes(st->dim, st->n_bins, tsize, a.hist_smem, a.edges_smem);
  const int64_t cap = (int64_t)sm_count() * TQ_SAMPLE_MIN_BLOCKS;  // resident CTAs
  // known point counts (warm-up): about two 32-point tiles per warp
  int64_t tiles = max_points > 0 ? (max_points + 2 * kTile - 1) / (2 * kTile) : cap;
  if (tiles > cap) tiles = cap;
  if (tiles < 1) tiles = 1;
  const dim3 grid((unsigned)tiles);
  if (st->dtype == TQ_F32 && st->dim <= 8)
    return launch_sample_f32_dims(a, family, st->dim, warm, grid.x, smem, s);
#define TQ_SAMPLE_LAUNCH(T, WARMB)                                                          \
  {                                                                                         \
    auto kfn = vegas_sample_kernel<T, FAM, WARMB, 0>;                                       \
    if (smem > 48 * 1024) {                                                                 \
      cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                           (int)smem);                                      \
      if (e != cudaSuccess) return set_cuda_error(e);                                       \
    }                                                                                       \
    kfn<<<grid, kTile, smem, s>>>(a);                                                       \
  }
  TQ_DISPATCH_FAMILY(family, FAM, {
    if (st->dtype == TQ_F64) {
      if (warm) TQ_SAMPLE_LAUNCH(double, true) else TQ_SAMPLE_LAUNCH(double, false)
    } else {
      if (warm) TQ_SAMPLE_LAUNCH(float, true) else TQ_SAMPLE_LAUNCH(float, false)
    }
  });
#undef TQ_SAMPLE_LAUNCH
  return launch_status();
}

extern "C" int tq_vegas_set_control(const tq_vegas_state* st, int mask, int64_t nevals_exp,
                                    int64_t slot, int64_t normalize, uint64_t seed,
                                    uint64_t stream_id, void* stream) {
  const int rc = check_state(st);
  if (rc != TQ_OK) return rc;
  if ((mask & TQ_VC_NEVALS) && nevals_exp < 0) return TQ_ERR_ARG;
  vegas_set_control_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(st->control, mask, nevals_exp, slot,
                                                              normalize, seed, stream_id);
  return launch_status();
}

extern "C" int tq_vegas_warmup_fused(const tq_vegas_state* st, int family, const double* params,
                                     int64_t n_samples, void* workspace, size_t workspace_bytes,
                                     void* stream) {
  TQ_VEGAS_WS();
  if (!params || n_samples < 1) return TQ_ERR_ARG;
  return launch_sample(st, family, params, n_samples, 1, n_samples, true, ws.t_sample, nullptr, s);
}

extern "C" int tq_vegas_iterate_fused(const tq_vegas_state* st, int family, const double* params,
                                      int use_grid_improve, int64_t max_points, void* workspace,
                                      size_t workspace_bytes, void* stream) {
  TQ_VEGAS_WS();
  if (!params || max_points < 0) return TQ_ERR_ARG;
  return launch_sample(st, family, params, 0, use_grid_improve ? 1 : 0, max_points, false,
                       ws.t_sample, ws.block_tot, s);
}

static int launch_update_map(const tq_vegas_state* st, double alpha, void* workspace,
                             size_t workspace_bytes, void* smooth_out, void* stream) {
  TQ_VEGAS_WS();
  if (st->n_bins > kSmallMap) {
    MapTiles m = map_tile_layout(st, ws.map_scratch);
    if (smooth_out) m.sw = smooth_out;
    const dim3 g((unsigned)map_tiles(st->n_bins), (unsigned)st->dim);
    const int sm_only = smooth_out ? 1 : 0;
#define TQ_TILED_MAP(T)                                                                 \
  {                                                                                     \
    map_fill_kernel<T><<<g, kMapThreads, 0, s>>>(*st, m, ws.t_map);                     \
    map_smooth_kernel<T><<<g, kMapThreads, 0, s>>>(*st, m, alpha, sm_only, ws.t_map + 4); \
    if (!sm_only) {                                                                     \
      map_multiples_kernel<T><<<g, kMapThreads, 0, s>>>(*st, m);                        \
      map_runs_kernel<T><<<g, kMapThreads, 0, s>>>(*st, m);                             \
      map_accu_sums_kernel<T><<<g, kMapThreads, 0, s>>>(*st, m, ws.t_map + 8);          \
      map_edges_kernel<T><<<g, kMapThreads, 0, s>>>(*st, m);                            \
      map_commit_kernel<T><<<g, kMapThreads, 0, s>>>(*st, m);                           \
    }                                                                                   \
  }
    if (st->dtype == TQ_F64)
      TQ_TILED_MAP(double)
    else
      TQ_TILED_MAP(float)
#undef TQ_TILED_MAP
    return launch_status();
  }
  const size_t smem = map_row_smem(st->n_bins, dtype_size(st->dtype));
#define TQ_ROWS_LAUNCH(T)                                                                      \
  {                                                                                            \
    auto kfn = vegas_map_rows_kernel<T>;                                                       \
    if (smem > 48 * 1024) {                                                                    \
      cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                           (int)smem);                                         \
      if (e != cudaSuccess) return set_cuda_error(e);                                          \
    }                                                                                          \
    kfn<<<st->dim, kRowThreads, smem, s>>>(*st, alpha, smooth_out, ws.t_map);                  \
  }
  if (st->dtype == TQ_F64) {
    TQ_ROWS_LAUNCH(double)
  } else {
    auto kfn = vegas_map_rows_f32_kernel;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return set_cuda_error(e);
    }
    kfn<<<st->dim, kRowThreads, smem, s>>>(*st, alpha, smooth_out, ws.t_map);
  }
#undef TQ_ROWS_LAUNCH
  return launch_status();
}

extern "C" int tq_vegas_update_map(const tq_vegas_state* st, double alpha, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  return launch_update_map(st, alpha, workspace, workspace_bytes, nullptr, stream);
}

extern "C" int tq_vegas_smooth_weights(const tq_vegas_state* st, double alpha, void* smoothed,
                                       void* workspace, size_t workspace_bytes, void* stream) {
  if (!smoothed) return TQ_ERR_ARG;
  return launch_update_map(st, alpha, workspace, workspace_bytes, smoothed, stream);
}

static int launch_nh(const tq_vegas_state* st, void* workspace, size_t workspace_bytes,
                     void* stream, bool split) {
  TQ_VEGAS_WS();
  NhArgs a;
  a.st = *st;
  a.block_tot = ws.block_tot;
  a.ticket = ws.t_nh;
  a.split = split ? 1 : 0;
  const unsigned g = (unsigned)nh_blocks(st);
  if (st->dtype == TQ_F64)
    vegas_nh_kernel<double><<<g, kBlock, 0, s>>>(a);
  else
    vegas_nh_kernel<float><<<g, kBlock, 0, s>>>(a);
  int e = launch_status();
  if (e != TQ_OK || split) return e;
  vegas_nh_fixup_kernel<<<g, kBlock, 0, s>>>(*st, ws.block_tot);
  return launch_status();
}

extern "C" int tq_vegas_get_nh(const tq_vegas_state* st, void* workspace, size_t workspace_bytes,
                               void* stream) {
  return launch_nh(st, workspace, workspace_bytes, stream, false);
}

extern "C" int tq_vegas_get_nh_split(const tq_vegas_state* st, void* workspace,
                                     size_t workspace_bytes, void* stream) {
  return launch_nh(st, workspace, workspace_bytes, stream, true);
}

extern "C" int tq_vegas_finish_iteration(const tq_vegas_state* st, double beta, void* workspace,
                                         size_t workspace_bytes, void* stream) {
  TQ_VEGAS_WS();
  FinishArgs a;
  a.st = *st;
  a.beta = beta;
  a.V = pow(1.0 / (double)st->n_strat, (double)st->dim);
  a.partials = ws.partials;
  a.ticket = ws.t_finish;
  a.block_pre = ws.block_tot;
  const unsigned g = (unsigned)finish_blocks(st);
  if (st->dtype == TQ_F64)
    vegas_finish_kernel<double><<<g, kBlock, 0, s>>>(a);
  else
    vegas_finish_f32_kernel<<<g, kBlock, 0, s>>>(a);
  return launch_status();
}

extern "C" int tq_vegas_finish_update_map(const tq_vegas_state* st, double beta, double alpha,
                                          void* workspace, size_t workspace_bytes, void* stream) {
  if (st && st->n_bins > kSmallMap) {
    const int rc = tq_vegas_finish_iteration(st, beta, workspace, workspace_bytes, stream);
    if (rc != TQ_OK) return rc;
    return tq_vegas_update_map(st, alpha, workspace, workspace_bytes, stream);
  }
  TQ_VEGAS_WS();
  FinishArgs a;
  a.st = *st;
  a.beta = beta;
  a.V = pow(1.0 / (double)st->n_strat, (double)st->dim);
  a.partials = ws.partials;
  a.ticket = ws.t_finish;
  a.block_pre = ws.block_tot;
  const unsigned g = (unsigned)finish_blocks(st) + (unsigned)st->dim;
  const size_t smem = map_row_smem(st->n_bins, dtype_size(st->dtype));
#define TQ_FINISH_MAP(T)                                                                      \
  {                                                                                           \
    auto kfn = vegas_finish_map_kernel<T>;                                                    \
    if (smem > 48 * 1024) {                                                                   \
      cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                           (int)smem);                                        \
      if (e != cudaSuccess) return set_cuda_error(e);                                         \
    }                                                                                         \
    kfn<<<g, kBlock, smem, s>>>(a, alpha, ws.t_map);                                          \
  }
  if (st->dtype == TQ_F64)
    TQ_FINISH_MAP(double)
  else
    TQ_FINISH_MAP(float)
#undef TQ_FINISH_MAP
  return launch_status();
}

static unsigned elem_grid(int64_t n) {
  int64_t g = (n + kTile - 1) / kTile;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (g > cap) g = cap;
  return (unsigned)(g < 1 ? 1 : g);
}

extern "C" int tq_vegas_strat_points(const tq_vegas_state* st, const void* u, int64_t n_points,
                                     void* y, void* stream) {
  const int rc = check_state(st);
  if (rc != TQ_OK) return rc;
  if (n_points < 0 || (n_points > 0 && (!u || !y))) return TQ_ERR_ARG;
  if (n_points == 0) return TQ_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (st->dtype == TQ_F64)
    vegas_strat_points_kernel<double><<<elem_grid(n_points), kTile, 0, s>>>(*st, (const double*)u, n_points, (double*)y);
  else
    vegas_strat_points_kernel<float><<<elem_grid(n_points), kTile, 0, s>>>(*st, (const float*)u, n_points, (float*)y);
  return launch_status();
}

extern "C" int tq_vegas_map_points(const tq_vegas_state* st, const void* y, int64_t n_points,
                                   void* x, void* jac, void* stream) {
  const int rc = check_state(st);
  if (rc != TQ_OK) return rc;
  if (n_points < 0 || (n_points > 0 && (!y || !x || !jac))) return TQ_ERR_ARG;
  if (n_points == 0) return TQ_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (st->dtype == TQ_F64)
    vegas_map_points_kernel<double><<<elem_grid(n_points), kTile, 0, s>>>(*st, (const double*)y, n_points, (double*)x, (double*)jac);
  else
    vegas_map_points_kernel<float><<<elem_grid(n_points), kTile, 0, s>>>(*st, (const float*)y, n_points, (float*)x, (float*)jac);
  return launch_status();
}

extern "C" int tq_vegas_accumulate(const tq_vegas_state* st, const void* y, const void* jf,
                                   int64_t n_points, int accumulate_map, int stratified,
                                   void* workspace, size_t workspace_bytes, void* stream) {
  TQ_VEGAS_WS();
  (void)ws;
  if (n_points < 0 || (n_points > 0 && (!y || !jf))) return TQ_ERR_ARG;
  if (n_points == 0) return TQ_OK;
  if (st->dtype == TQ_F64)
    vegas_accumulate_kernel<double><<<elem_grid(n_points), kTile, 0, s>>>(*st, (const double*)y, (const double*)jf, n_points, accumulate_map, stratified);
  else
    vegas_accumulate_kernel<float><<<elem_grid(n_points), kTile, 0, s>>>(*st, (const float*)y, (const float*)jf, n_points, accumulate_map, stratified);
  return launch_status();
}
