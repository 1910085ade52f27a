// VEGAS+ on GB300: fused stratified sampling (Philox -> stratified y ->
// adaptive-map x, jac -> integrand -> map histogram and per-cube sums), the
// map update and the stratification update.
//
// Reference (torchquad v0.5.0): vegas.py (driver), vegas_map.py (adaptive
// map), vegas_stratification.py (stratified sampling).  The reference
// materialises y, x, f and jac for every point and scatter-adds them into
// the map and the cubes with global atomics (utils.py:61-76).  Here one
// kernel does a whole iteration: each warp takes 32 consecutive points,
// generates them in registers, adds to a warp-private map histogram in
// shared memory (lanes hitting the same interval are combined first, so the
// adds are plain and their order fixed), and reduces the per-cube sums with
// a segmented scan over the cube-contiguous point order (repeat_interleave
// order of vegas_stratification.py:154; a warp spans at most 17 cubes
// because every cube has >= 2 points) into one global add per cube segment.
// The histograms are flushed once per CTA.
//
// The arithmetic that decides interval indices and points (y, ID, offset,
// x, jac) is written with explicitly rounded operations in the state's
// dtype, in the reference's operation order, so that indices and counts
// match the reference bit for bit given the same uniforms and map.

#pragma once

#include <type_traits>

#include "tq_common.cuh"

namespace tq {

constexpr int kTile = 256;  // threads per CTA of the sampler
#ifndef TQ_SAMPLE_MIN_BLOCKS
#define TQ_SAMPLE_MIN_BLOCKS 4  // resident sampler CTAs per SM (64 registers)
#endif

// ---- explicitly rounded arithmetic (no FMA contraction)
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

template <typename T>
__device__ __forceinline__ T warm_scale() {
  return (T)0.999999;  // vegas.py:236 (and the clamp of vegas_stratification.py:165)
}

// Map one coordinate: interval ID = floor(y*B), offset = y*B - floor(y*B)
// (vegas_map.py:76-97), x = x_edges[ID] + dx_edges[ID]*offset (:57),
// Jacobian factor B * dx_edges[ID] (:73).
template <typename T>
__device__ __forceinline__ int map_coord(const T* __restrict__ xe, const T* __restrict__ dxe,
                                         int B, T Bf, T y, T& x, T& jac_factor) {
  const T yB = mul_rn(y, Bf);
  const T fl = floor(yB);
  int id = (int)fl;
  // y < 1 keeps id <= B-1; the clamp only guards memory for pathological B
  id = id < 0 ? 0 : (id >= B ? B - 1 : id);
  const T off = sub_rn(yB, fl);
  x = add_rn(xe[id], mul_rn(dxe[id], off));
  jac_factor = mul_rn(Bf, dxe[id]);
  return id;
}

// Coordinate k of the position of cube c: (c / n_strat^k) mod n_strat,
// dimension 0 fastest (vegas_stratification.py:105-138).
__device__ __forceinline__ int64_t cube_digit(int64_t c, int64_t n_strat, int k) {
  for (int i = 0; i < k; ++i) c /= n_strat;
  return c % n_strat;
}

// y = (pos + u) / n_strat, values >= 1 replaced by 0.999999 (:159-165).
// pos < n_strat < 2^31: 32-bit conversion.
template <typename T>
__device__ __forceinline__ T strat_y(int pos, T u, T nsf) {
  T y = div_rn(add_rn((T)pos, u), nsf);
  return y >= (T)1 ? warm_scale<T>() : y;
}

// cube_start[c] for c < n_cubes; pre != nullptr: cube_start is split
// (kCtlSplit) and pre holds the offsets of its kBlock-cube blocks.  Both
// are read-only for the lifetime of a sampling launch (get_NH and finish,
// which write them, are launches of their own), so the loads take the
// read-only data path.
__device__ __forceinline__ int64_t cube_start_at(const int64_t* cs, const int64_t* pre, int64_t c) {
  return pre ? __ldg(cs + c) + __ldg(pre + c / kBlock) : __ldg(cs + c);
}

// Largest c in [0, n) with cube_start[c] <= target; strictly increasing,
// cube_start[0] = 0.  One warp, 32-ary search with coalesced probes.
__device__ __forceinline__ int64_t warp_find_cube(const int64_t* cs, const int64_t* pre, int64_t n,
                                                  int64_t target) {
  const int lane = threadIdx.x & 31;
  int64_t lo = 0, hi = n;
  while (hi - lo > 32) {
    const int64_t step = (hi - lo + 31) / 32;
    const int64_t pos = lo + lane * step;
    const bool ok = pos < hi && cube_start_at(cs, pre, pos) <= target;
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    const int last = 31 - __clz(m);
    lo = lo + last * step;
    hi = min(hi, lo + step);
  }
  const int64_t pos = lo + lane;
  const bool ok = pos < hi && cube_start_at(cs, pre, pos) <= target;
  const unsigned m = __ballot_sync(0xffffffffu, ok);
  return lo + (31 - __clz(m));
}

// ------------------------------------------------------------ sampling
struct SampleArgs {
  tq_vegas_state st;
  int family;
  const double* params;
  int64_t n_samples;  // warm-up: points; iterations: read from cube_start
  int use_map;        // accumulate the map histogram
  int edges_smem, hist_smem;
  int small_cubes;    // n_cubes < 2^32: cube digits with 32-bit division
  FastDiv ns_div;     // division by n_strat
  unsigned* ticket;
  const int64_t* block_pre;  // block offsets of a split cube_start (kCtlSplit)
};

// Histogram weight type in shared memory: fp32 atomics are native, so the
// fp32 path privatises in fp32 and flushes once per CTA into fp64.
template <typename T>
struct HistT {
  using type = double;
};
template <>
struct HistT<float> {
  using type = float;
};

// Shared memory of the sampler: the map (edges) when it fits, and one
// private histogram per warp (weights in HistT, counts in u32) when it fits.
template <typename T>
struct Smem {
  T* xe;
  T* dxe;
  typename HistT<T>::type* hw;  // [warps][d*B]
  unsigned* hc;                 // [warps][d*B]
};

constexpr int kWarps = kTile / 32;

__host__ __device__ inline size_t sample_smem_bytes(int d, int64_t B, size_t tsize, bool hist,
                                                    bool edges) {
  size_t off = 0;
  if (edges) off += tsize * (d * (B + 1) + d * B);
  off = (off + 15) & ~size_t(15);
  if (hist) off += (size_t)kWarps * d * B * (tsize + sizeof(unsigned));  // HistT<T> weight, u32 count
  return off;
}

template <typename T>
__device__ Smem<T> carve(unsigned char* base, const SampleArgs& a) {
  Smem<T> s;
  const int d = a.st.dim;
  const int64_t B = a.st.n_bins;
  size_t off = 0;
  if (a.edges_smem) {
    s.xe = (T*)(base + off);
    off += sizeof(T) * d * (B + 1);
    s.dxe = (T*)(base + off);
    off += sizeof(T) * d * B;
  } else {
    s.xe = (T*)a.st.x_edges;
    s.dxe = (T*)a.st.dx_edges;
  }
  off = (off + 15) & ~size_t(15);
  if (a.hist_smem) {
    s.hw = (typename HistT<T>::type*)(base + off);
    off += (size_t)kWarps * d * B * sizeof(typename HistT<T>::type);
    s.hc = (unsigned*)(base + off);
  } else {
    s.hw = nullptr;
    s.hc = nullptr;
  }
  return s;
}

// Warp-private histogram update without atomics: lanes with the same key
// form a group (__match_any_sync) and sum their values by pointer jumping
// along the group in lane order (ceil(log2(largest group)) shuffle steps: a
// fixed tree, so the result does not depend on scheduling); the group's
// lowest lane then adds the sum and the group's size to the bin.  Groups
// have distinct keys, so no two lanes write one bin.  Stratified points of a
// tile share cubes, so groups of 8 or more lanes are common.  The caller
// orders successive calls on the same bins with __syncwarp().
template <typename H>
__device__ __forceinline__ void warp_hist_add(H* hw, unsigned* hc, int key, bool valid, H v) {
  const int lane = threadIdx.x & 31;
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  const unsigned above = grp & ~((2u << lane) - 1u);  // members after this lane
  int nxt = above ? __ffs(above) - 1 : 32;
  const unsigned size = (unsigned)__popc(grp);
  const unsigned largest = __reduce_max_sync(0xffffffffu, valid ? size : 1u);
  for (unsigned span = 1; span < largest; span <<= 1) {
    const H w = __shfl_sync(0xffffffffu, v, nxt & 31);
    const int n2 = __shfl_sync(0xffffffffu, nxt, nxt & 31);
    if (nxt < 32) {
      v += w;
      nxt = n2;
    }
  }
  if (valid && (grp & ((1u << lane) - 1u)) == 0u) {
    hw[key] += v;
    hc[key] += size;
  }
}

// The integrand inside the sampler with every rounding spelled out (the
// products of the separable sum fused into its adds, one rounding each), so
// that the dimension-specialised, the generic and the batched samplers
// compute the same values whatever the compiler would contract.
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// s + g_k(x) (g_0(x) for k = 0).
template <int FAM, typename T>
__device__ __forceinline__ T vegas_sum(const Family<T>& f, int k, T x, T s) {
  if (FAM == TQ_FN_GAUSSIAN) {
    const T d = sub_rn(x, f.u[k]);
    const T dd = mul_rn(d, d);
    return k == 0 ? mul_rn(f.a[k], dd) : fma_rn(f.a[k], dd, s);
  } else if (FAM == TQ_FN_SUM_SIN) {
    const T g = sin(mul_rn(f.a[k], x));
    return k == 0 ? g : add_rn(s, g);
  } else {
    return k == 0 ? mul_rn(f.a[k], x) : fma_rn(f.a[k], x, s);
  }
}
template <int FAM, typename T>
__device__ __forceinline__ T vegas_outer(const Family<T>& f, T s) {
  if (FAM == TQ_FN_EXP_SUM) return mul_rn(f.c, exp(add_rn(s, f.b)));
  if (FAM == TQ_FN_GAUSSIAN) return mul_rn(f.c, exp(-s));
  if (FAM == TQ_FN_OSCILLATORY) return mul_rn(f.c, cos(fma_rn((T)(2.0 * CUDART_PI), f.b, s)));
  return mul_rn(f.c, s);  // TQ_FN_SUM_SIN
}

// Philox blocks a point's D draws can touch: a point's first draw sits at
// word (j*D) mod PB of its first block, at most PB - gcd(D, PB).
__host__ __device__ constexpr int gcd_c(int a, int b) { return b == 0 ? a : gcd_c(b, a % b); }
template <int D, int PB>
struct DrawBlocks {
  static constexpr int step = gcd_c(D, PB);               // first-word offsets are multiples
  static constexpr int blocks = (PB - step + D + PB - 1) / PB;
};

// D > 0: the dimension is known at compile time (fully unrolled point
// loops, D interval indices in registers); D = 0: any dimension up to
// kMaxDim from the state.
// The sampler as a device body: CTA bid of nblk CTAs taking part (the
// per-launch kernel below, or one state's share of a batched launch).
template <typename T, int FAM, bool WARM, int D>
__device__ void sample_body(const SampleArgs& a, unsigned bid, unsigned nblk) {
  constexpr int KD = D > 0 ? D : kMaxDim;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Family<T> fam;
  __shared__ T lo[kMaxDim], wid[kMaxDim];
  __shared__ T volume;
  using H = typename HistT<T>::type;  // fp32 on the fp32 path
  const tq_vegas_state& st = a.st;
  const int d = D > 0 ? D : st.dim;
  const int64_t B = st.n_bins;
  const int64_t DB = d * B;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Smem<T> sm = carve<T>(smem_raw, a);
  if (threadIdx.x == 0) {
    load_family<T>(fam, a.family, d, a.params);
    const T* dom = (const T*)st.domain;
    T v = (T)1;
    for (int k = 0; k < d; ++k) {
      lo[k] = dom[2 * k];
      wid[k] = sub_rn(dom[2 * k + 1], dom[2 * k]);
      v = mul_rn(v, wid[k]);
    }
    volume = v;
  }
  if (a.edges_smem) {
    for (int64_t i = threadIdx.x; i < d * (B + 1); i += blockDim.x) sm.xe[i] = ((const T*)st.x_edges)[i];
    for (int64_t i = threadIdx.x; i < DB; i += blockDim.x) sm.dxe[i] = ((const T*)st.dx_edges)[i];
  }
  if (a.hist_smem) {
    for (int64_t i = threadIdx.x; i < (int64_t)kWarps * DB; i += blockDim.x) {
      sm.hw[i] = 0;
      sm.hc[i] = 0u;
    }
  }

  const int64_t M = WARM ? a.n_samples : __ldcg(st.cube_start + st.n_cubes);
  const uint64_t offset = *st.rng_offset;
  const uint64_t seed = (uint64_t)st.control[3], sid = (uint64_t)st.control[4];
  const int64_t ns = st.n_strat;
  const T nsf = (T)ns;
  const int Bi = (int)B;
  const T Bf = (T)Bi;
  constexpr int PB = Uniform<T>::per_block;

  // Warp tiles of 32 consecutive points; every cube has >= 2 points, so a
  // tile spans at most 17 cubes.  Each warp takes a contiguous range of
  // tiles (balanced to one tile), finds the cube of its first point once and
  // then walks the cube boundaries tile by tile.  The search (dependent
  // global loads) runs before the barrier, beside the loads of the map and
  // the integrand parameters.
  const int64_t n_tiles = (M + 31) / 32;
  const int64_t n_warps = (int64_t)nblk * kWarps;
  const int64_t gw = (int64_t)bid * kWarps + warp;
  const int64_t t_begin = gw * n_tiles / n_warps, t_end = (gw + 1) * n_tiles / n_warps;
  int64_t c0 = 0;  // cube of the tile's first point
  const int64_t* pre = (!WARM && st.control[kCtlSplit] != 0) ? a.block_pre : nullptr;
  if (!WARM && t_begin < t_end) c0 = warp_find_cube(st.cube_start, pre, st.n_cubes, t_begin * 32);
  __syncthreads();
  H* whw = a.hist_smem ? sm.hw + warp * DB : nullptr;
  unsigned* whc = a.hist_smem ? sm.hc + warp * DB : nullptr;
  for (int64_t wt = t_begin; wt < t_end; ++wt) {
    const int64_t j0 = wt * 32;
    const int64_t j = j0 + lane;
    const bool valid = j < M;
    int slot = -1;
    int64_t csl = 0;
    unsigned starts = 0u;
    if (!WARM) {
      const int64_t cl = c0 + lane;
      csl = cl < st.n_cubes ? cube_start_at(st.cube_start, pre, cl)
                            : (cl == st.n_cubes ? __ldg(st.cube_start + cl) : INT64_MAX);
      // bit p: a cube starts at point j0 + p (cube c0 holds j0, so the
      // starts of cubes c0 + 1.. lie after j0); the slot of point j0 + p
      // (largest l with cube_start[c0 + l] <= j) counts the starts in bits 1..p
      const int64_t off = csl - j0;
      const unsigned bit = (off > 0 && off < 32) ? (1u << (int)off) : 0u;
      starts = __reduce_or_sync(0xffffffffu, bit);
      slot = valid ? __popc(starts & ((2u << lane) - 1u)) : -1;
    }
    H jfd = 0, jf2 = 0;
    int ids[KD];
    if (valid) {
      uint32_t c32 = (uint32_t)(c0 + slot);
      uint64_t c = (uint64_t)(c0 + slot);
      // Philox block of this point's first draw; later draws follow
      const uint64_t e0 = (uint64_t)j * (uint64_t)d;
      const uint64_t blk0 = offset + e0 / PB;
      const int lane0 = (int)(e0 % PB);
      int cur = -1;
      uint4 r = make_uint4(0, 0, 0, 0);
      // fp32 with the dimension fixed: every lane computes the blocks its
      // draws can touch at once (no divergent per-draw block branch) and
      // picks its words by its first word's offset
      constexpr bool kWords = std::is_same<T, float>::value && D > 0;
      constexpr int NB = kWords ? DrawBlocks<(D > 0 ? D : 1), PB>::blocks : 1;
      constexpr int GS = kWords ? DrawBlocks<(D > 0 ? D : 1), PB>::step : 1;
      uint32_t words[4 * NB];
      if constexpr (kWords) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          const uint4 rb = philox_block(seed, sid, blk0 + (uint64_t)b);
          words[4 * b] = rb.x;
          words[4 * b + 1] = rb.y;
          words[4 * b + 2] = rb.z;
          words[4 * b + 3] = rb.w;
        }
      }
      T jac = (T)1;
      T s = T(0);
#pragma unroll
      for (int k = 0; k < KD; ++k) {
        if (k < d) {
          T u;
          if constexpr (kWords) {
            uint32_t w = words[k];
#pragma unroll
            for (int o = GS; o < PB; o += GS)
              if (k + o < 4 * NB) w = lane0 == o ? words[k + o] : w;
            u = (T)u32_to_unit_f(w);
          } else {
            const int le = lane0 + k;
            const int bi = le / PB;
            if (bi != cur) {
              r = philox_block(seed, sid, blk0 + (uint64_t)bi);
              cur = bi;
            }
            u = Uniform<T>::from(r, le - bi * PB);
          }
          T y;
          if (WARM) {
            y = mul_rn(u, warm_scale<T>());
          } else {
            int pos;
            if (a.small_cubes) {
              const uint32_t q = fdiv(c32, a.ns_div);
              pos = (int)(c32 - q * a.ns_div.d);
              c32 = q;
            } else {
              const uint64_t q = c / (uint64_t)ns;
              pos = (int)(c - q * (uint64_t)ns);
              c = q;
            }
            y = strat_y<T>(pos, u, nsf);
          }
          T x, jf_k;
          ids[k] = map_coord<T>(sm.xe + k * (Bi + 1), sm.dxe + k * Bi, Bi, Bf, y, x, jf_k);
          jac = mul_rn(jac, jf_k);
          // vegas.py:110: fn(x * domain_sizes + domain_starts) * domain_volume
          const T xt = add_rn(mul_rn(x, wid[k]), lo[k]);
          s = vegas_sum<FAM, T>(fam, k, xt, s);
        }
      }
      const T f = mul_rn(vegas_outer<FAM, T>(fam, s), volume);
      const T jfv = mul_rn(f, jac);
      jfd = (H)jfv;
      jf2 = jfd * jfd;
    }
    if (a.use_map) {
#pragma unroll
      for (int k = 0; k < KD; ++k) {
        if (k < d) {
          if (a.hist_smem) {
            const int key = valid ? (int)(k * B) + ids[k] : -1 - lane;
            warp_hist_add<H>(whw, whc, key, valid, jf2);
          } else if (valid) {
            atomicAdd(st.weights + k * B + ids[k], (double)jf2);
            atomicAdd((unsigned long long*)(st.counts + k * B + ids[k]), 1ull);
          }
        }
      }
      if (a.hist_smem) __syncwarp();  // the next tile's groups may differ
    }
    if (!WARM) {
      // points are in cube order: segmented inclusive scan over the warp,
      // then one global add per cube segment
      // lane's segment starts at the last cube start at or before it
      const unsigned upto = starts & ((2u << lane) - 1u);
      const int head = upto ? 31 - __clz(upto) : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const H a1 = __shfl_up_sync(0xffffffffu, jfd, o);
        const H a2 = __shfl_up_sync(0xffffffffu, jf2, o);
        if (lane - o >= head) {
          jfd += a1;
          jf2 += a2;
        }
      }
      // segment end: a cube starts at the next point, or this is the last
      const bool seg_end = lane == 31 || (((starts >> 1) >> lane) & 1u) != 0u || j + 1 >= M;
      if (slot >= 0 && seg_end) {
        atomicAdd(st.jf + c0 + slot, (double)jfd);
        atomicAdd(st.jf2 + c0 + slot, (double)jf2);
      }
      // cube of the next tile's first point (at most 17 cubes ahead)
      const unsigned ahead = __ballot_sync(0xffffffffu, csl <= j0 + 32);
      c0 += 31 - __clz(ahead);
    }
  }
  if (a.hist_smem && a.use_map) {
    __syncthreads();
    for (int64_t i = threadIdx.x; i < DB; i += blockDim.x) {
      unsigned cnt = 0;
      H w = 0;
#pragma unroll
      for (int q = 0; q < kWarps; ++q) {
        cnt += sm.hc[q * DB + i];
        w += sm.hw[q * DB + i];
      }
      if (cnt) {
        atomicAdd(st.weights + i, (double)w);
        atomicAdd((unsigned long long*)(st.counts + i), (unsigned long long)cnt);
      }
    }
  }
  // The last CTA advances the RNG offset.  It reads nothing the other CTAs
  // wrote (each read the offset before taking its ticket), so no fence.
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(a.ticket, 1u) == nblk - 1) {
    *st.rng_offset = offset + ((uint64_t)M * d + PB - 1) / PB;
    *a.ticket = 0u;
  }
}

template <typename T, int FAM, bool WARM, int D>
__global__ void __launch_bounds__(kTile, TQ_SAMPLE_MIN_BLOCKS) vegas_sample_kernel(SampleArgs a) {
  sample_body<T, FAM, WARM, D>(a, blockIdx.x, gridDim.x);
}

// fp32 states with 1 <= dim <= 8: the dimension-specialised sampler
// (tq_vegas_sample_d.cu), iterations and warm-up.
int launch_sample_f32_dims(const SampleArgs& a, int family, int dim, bool warm, unsigned grid,
                           size_t smem, cudaStream_t s);

}  // namespace tq
