// Phases of a VEGAS iteration as device bodies, shared by the per-phase
// kernels of one state (tq_vegas.cu) and the kernels that advance many
// states per launch (tq_vegas_batch.cu): get_NH, the end of an iteration
// (estimate, variance, update_DH), the map update of maps of at most
// kSmallMap intervals, and the state reset.  Each body takes its CTA index
// and the number of CTAs that share the phase.
//
// Reference (torchquad v0.5.0): vegas.py (driver), vegas_map.py (adaptive
// map), vegas_stratification.py (stratified sampling).
#pragma once

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
static __device__ void nh_body(const NhArgs& a, unsigned bid, unsigned nblk) {
  const tq_vegas_state& st = a.st;
  const int64_t c = (int64_t)bid * blockDim.x + threadIdx.x;
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
  if (threadIdx.x == 0) a.block_tot[bid] = warp_tot[kBlock / 32 - 1];
  if (last_block_of(a.ticket, nblk)) {
    // exclusive scan of the block totals, kBlock at a time
    int64_t carry = 0;
    for (unsigned base = 0; base < nblk; base += kBlock) {
      const unsigned b = base + threadIdx.x;
      const int64_t t = b < nblk ? a.block_tot[b] : 0;
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
      if (b < nblk) a.block_tot[b] = ex;
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
static __device__ __forceinline__ void block_sum3(double& x, double& y, double& z, double* sh) {
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
static __device__ void finish_body(const FinishArgs& a, unsigned bid, unsigned nblk) {
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


// fp32 states: the per-cube terms in fp32 (the reference computes them in
// the state's dtype), every sum as a double-float on the FP32 pipe: per
// thread, over the CTA, and across CTAs in the last one.  The only FP64
// instructions are the two conversions of the cube's fp64 sums per cube.
static __device__ __forceinline__ void f2_warp_sum3(F2& x, F2& y, F2& z) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const F2 x2 = f2_shfl_down(x, o), y2 = f2_shfl_down(y, o), z2 = f2_shfl_down(z, o);
    x = f2_add(x, x2);
    y = f2_add(y, y2);
    z = f2_add(z, z2);
  }
}

static __device__ void finish_f32_body(const FinishArgs& a, unsigned bid, unsigned nblk) {
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


// --------------------------------------------------------- map update
// Block-wide sum (fp64), result in every thread.
static __device__ double block_sum_all(double v, double* sh) {
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

// Exclusive scan of one value per thread across the CTA (fixed order).
static __device__ __forceinline__ double cta_exclusive_scan(double x, double* sh) {
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
static __device__ void clear_map_by_last(const tq_vegas_state& st, unsigned* ticket, unsigned nrows) {
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
static __device__ void map_rows_body(const tq_vegas_state& st, double alpha, void* smooth_out, unsigned* ticket,
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
  // zero-row test over the whole map; a row's remaining averages are
  // skipped once some thread has found a nonzero one (the flag only ever
  // goes from 0 to 1, so the outcome is the same)
  if (threadIdx.x < d) rownz[threadIdx.x] = 0;
  __syncthreads();
  volatile int* rnz = rownz;
  for (int kk = 0; kk < d; ++kk) {
    for (int b = threadIdx.x; b < B && !rnz[kk]; b += blockDim.x) {
      const int64_t c = st.counts[(int64_t)kk * B + b];
      const T wi = (T)st.weights[(int64_t)kk * B + b];
      if ((c == 0 ? wi : div_rn(wi, (T)c)) != (T)0) rnz[kk] = 1;
    }
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


// fp32 maps: the same update with every fp64 sum and scan of the generic
// kernel as a double-float on the FP32 pipe (the reference's fp64
// cumulative sums of fp32 values are exact in both forms whenever they are
// exact in fp64).  The delta multiple of a cumulative sum C = hi + lo is the
// largest k with k * delta <= C, decided from the exact residual (k * delta
// as a TwoProduct): multiples agree with the fp64 truncation except where
// C / delta lies within about 2^-46 of an integer without being one.
static __device__ F2 f2_block_sum_all(F2 v, F2* sh) {
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

static __device__ F2 f2_cta_exclusive_scan(F2 x, F2* sh) {
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
static __device__ __forceinline__ bool f2_at_least(F2 c, int k, float delta) {
  const float kf = (float)k;
  const float ph = __fmul_rn(kf, delta);
  const float pl = __fmaf_rn(kf, delta, -ph);  // k * delta = ph + pl exactly
  const float r = __fsub_rn(__fadd_rn(__fsub_rn(c.hi, ph), c.lo), pl);
  return r >= 0.f;
}

static __device__ void map_rows_f32_body(const tq_vegas_state& st, double alpha, void* smooth_out, unsigned* ticket,
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
  volatile int* rnz = rownz;  // other rows: skipped once found nonzero (0 -> 1 only)
  for (int i = threadIdx.x; i < d * B; i += blockDim.x) {
    const int kk = i / B, b = i - kk * B;
    if (kk != k && rnz[kk]) continue;
    const int64_t c = st.counts[i];
    const T wi = (T)st.weights[i];
    const T av = c == 0 ? wi : div_rn(wi, (T)c);
    if (av != (T)0) rnz[kk] = 1;
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


// finish_iteration and update_map in one launch (maps of at most kSmallMap
// intervals): CTAs 0..d-1 update the map rows, the others end the
// iteration.  The two read and write disjoint parts of the state, so they
// run side by side; each role counts its own CTAs on its own ticket.

// ----------------------------------------------------------- init
template <typename T>
static __device__ void init_body(const tq_vegas_state& st, unsigned bid, unsigned nblk) {
  const int d = st.dim;
  const int64_t B = st.n_bins;
  const T step = div_rn((T)1, (T)B);  // linspace(0, 1, B+1) step
  for (int64_t i = (int64_t)bid * blockDim.x + threadIdx.x; i < d * (B + 1);
       i += (int64_t)nblk * blockDim.x) {
    const int64_t b = i % (B + 1);
    ((T*)st.x_edges)[i] = linspace_node<T>((T)0, (T)1, step, B + 1, b);
  }
  const T inv = div_rn((T)1, (T)B);  // ones / N_intervals (vegas_map.py:34-37)
  for (int64_t i = (int64_t)bid * blockDim.x + threadIdx.x; i < d * B;
       i += (int64_t)nblk * blockDim.x) {
    ((T*)st.dx_edges)[i] = inv;
    st.weights[i] = 0.0;
    st.counts[i] = 0;
  }
  // dh = ones * 1.0 / N_cubes (vegas_stratification.py:40)
  const T dh0 = div_rn((T)1, (T)st.n_cubes);
  for (int64_t c = (int64_t)bid * blockDim.x + threadIdx.x; c < st.n_cubes;
       c += (int64_t)nblk * blockDim.x) {
    ((T*)st.dh)[c] = dh0;
    st.jf[c] = 0.0;
    st.jf2[c] = 0.0;
    st.neval[c] = 0;
  }
  if (bid == 0 && threadIdx.x < 4) {
    st.flags[threadIdx.x] = 0;
    st.scalars[threadIdx.x] = 0.0;
  }
  if (bid == 0 && threadIdx.x == 0) {
    st.control[1] = 0;
    st.control[2] = 0;
    st.control[kCtlSplit] = 0;
  }
}

// ------------------------------------------------------------ host side
// Shared with the batched launchers; defined in tq_vegas.cu.
int vegas_check_state(const tq_vegas_state* st);
int64_t vegas_nh_blocks(const tq_vegas_state* st);
int64_t vegas_finish_blocks(const tq_vegas_state* st);
// CTAs of a sampling launch sized for `points` points (at most one wave).
int64_t vegas_sample_ctas(const tq_vegas_state* st, int64_t points);
struct VegasWsView {
  unsigned* t_sample;
  unsigned* t_nh;
  unsigned* t_finish;
  unsigned* t_map;
  int64_t* block_tot;
  Acc* partials;
  size_t total;
};
VegasWsView vegas_workspace_view(const tq_vegas_state* st, void* base);
// The sampler's arguments and dynamic shared memory for a state; the map
// edges are copied to shared memory while the total stays within
// edges_limit bytes (a lone state affords 96 KB; a batch keeps its launch
// at four resident CTAs per SM).
SampleArgs vegas_sample_args(const tq_vegas_state* st, int family, const double* params, int64_t n_samples,
                             int use_map, unsigned* ticket, const int64_t* block_pre, size_t* smem,
                             size_t edges_limit = 96 * 1024);

}  // namespace tq
