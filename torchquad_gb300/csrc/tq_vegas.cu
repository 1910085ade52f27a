// VEGAS+ on GB300: the per-phase kernels (get_NH, the end of an iteration,
// the adaptive-map update, the state reset), the tiled update of large maps,
// the materialised-path kernels and the C-ABI entry points of the VEGAS
// state.  The phase bodies are in tq_vegas_phases.cuh, the fused sampler in
// tq_vegas_sample.cuh.
//
// Reference (torchquad v0.5.0): vegas.py (driver), vegas_map.py (adaptive
// map), vegas_stratification.py (stratified sampling).

#include <type_traits>

#include "tq_vegas_phases.cuh"

namespace tq {

// ------------------------------------------- per-phase kernels
template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_nh_kernel(NhArgs a) {
  nh_body<T>(a, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kBlock) vegas_nh_fixup_kernel(tq_vegas_state st,
                                                                const int64_t* block_pre) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < st.n_cubes) st.cube_start[c] += block_pre[blockIdx.x];
}

template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_finish_kernel(FinishArgs a) {
  finish_body<T>(a, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kBlock) vegas_finish_f32_kernel(FinishArgs a) {
  finish_f32_body(a, blockIdx.x, gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(kRowThreads) vegas_map_rows_kernel(tq_vegas_state st, double alpha,
                                                                      void* smooth_out, unsigned* ticket) {
  map_rows_body<T>(st, alpha, smooth_out, ticket, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kRowThreads) vegas_map_rows_f32_kernel(tq_vegas_state st, double alpha,
                                                                          void* smooth_out, unsigned* ticket) {
  map_rows_f32_body(st, alpha, smooth_out, ticket, blockIdx.x, gridDim.x);
}

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

template <typename T>
__global__ void vegas_init_kernel(tq_vegas_state st) {
  init_body<T>(st, blockIdx.x, gridDim.x);
}

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

namespace tq {
int vegas_check_state(const tq_vegas_state* st) { return check_state(st); }
int64_t vegas_nh_blocks(const tq_vegas_state* st) { return nh_blocks(st); }
int64_t vegas_finish_blocks(const tq_vegas_state* st) { return finish_blocks(st); }
int64_t vegas_sample_ctas(const tq_vegas_state*, int64_t points) {
  // Two 32-point tiles per warp.  Fatter CTAs would spend less on their own
  // copy of the map and their histograms (O(dim x intervals) to fill and
  // flush), but a lone state then waits on fewer, longer CTAs; a batch
  // sizes its states the same way, so each gets the CTA split (and the fp32
  // partial sums) of its own per-call run.
  const int64_t per = 2 * kTile;
  const int64_t cap = (int64_t)sm_count() * TQ_SAMPLE_MIN_BLOCKS;
  const int64_t c = (points + per - 1) / per;
  return c < 1 ? 1 : (c > cap ? cap : c);
}
VegasWsView vegas_workspace_view(const tq_vegas_state* st, void* base) {
  const VegasWs w = vegas_ws(st, base);
  VegasWsView v;
  v.t_sample = w.t_sample;
  v.t_nh = w.t_nh;
  v.t_finish = w.t_finish;
  v.t_map = w.t_map;
  v.block_tot = w.block_tot;
  v.partials = w.partials;
  v.total = w.total;
  return v;
}
SampleArgs vegas_sample_args(const tq_vegas_state* st, int family, const double* params, int64_t n_samples,
                             int use_map, unsigned* ticket, const int64_t* block_pre, size_t* smem,
                             size_t edges_limit) {
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
  // The histograms go to shared memory up to 48 KB whatever the launch (the
  // choice changes how the fp32 sums are grouped, so it depends on the state
  // alone); the map edges join them up to edges_limit in all.
  a.hist_smem = sample_smem_bytes(st->dim, st->n_bins, tsize, true, false) <= 48 * 1024 &&
                st->dim * st->n_bins < (int64_t(1) << 30);
  a.edges_smem = sample_smem_bytes(st->dim, st->n_bins, tsize, a.hist_smem, true) <= edges_limit;
  *smem = sample_smem_bytes(st->dim, st->n_bins, tsize, a.hist_smem, a.edges_smem);
  return a;
}
}  // namespace tq

static int launch_sample(const tq_vegas_state* st, int family, const double* params,
                         int64_t n_samples, int use_map, int64_t max_points, bool warm,
                         unsigned* ticket, const int64_t* block_pre, cudaStream_t s) {
  size_t smem = 0;
  SampleArgs a = vegas_sample_args(st, family, params, n_samples, use_map, ticket, block_pre, &smem);
  const int64_t cap = (int64_t)sm_count() * TQ_SAMPLE_MIN_BLOCKS;  // resident CTAs
  const dim3 grid((unsigned)(max_points > 0 ? vegas_sample_ctas(st, max_points) : cap));
  if (st->dtype == TQ_F32 && st->dim <= 8)
    return launch_sample_f32_dims(a, family, st->dim, warm, grid.x, smem, s);
#define TQ_SAMPLE_LAUNCH(T, WARMB)                                                          \
  {                                                                                         \
    auto kfn = vegas_sample_kernel<T, FAM, WARMB, 0>;                                       \
    { const int orc = opt_in_smem(kfn, smem); if (orc != TQ_OK) return orc; }                   \
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
    { const int orc = opt_in_smem(kfn, smem); if (orc != TQ_OK) return orc; }                   \
    kfn<<<st->dim, kRowThreads, smem, s>>>(*st, alpha, smooth_out, ws.t_map);                  \
  }
  if (st->dtype == TQ_F64) {
    TQ_ROWS_LAUNCH(double)
  } else {
    auto kfn = vegas_map_rows_f32_kernel;
    {
      const int orc = opt_in_smem(kfn, smem);
      if (orc != TQ_OK) return orc;
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
    { const int orc = opt_in_smem(kfn, smem); if (orc != TQ_OK) return orc; }                   \
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
