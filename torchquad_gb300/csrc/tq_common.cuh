// Shared device code of the torchquad_gb300 kernels: status plumbing,
// compensated accumulators, Philox4x32-10, node/weight formulas of the grid
// rules and the built-in integrand families.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "torchquad_gb300.h"

namespace tq {

constexpr int kMaxDim = TQ_MAX_DIM;
constexpr int kBlock = 256;  // threads per CTA of the streaming kernels
// VEGAS control block entry: 1 while cube_start holds prefixes local to each
// kBlock-cube block of get_NH, the block offsets being in the workspace
// (tq_vegas_get_nh_split); the sampler adds them, finish writes them back.
constexpr int kCtlSplit = 14;

// ---------------------------------------------------------------- host side
int set_cuda_error(cudaError_t e);  // records e, returns TQ_ERR_CUDA
int launch_status();                // TQ_OK or TQ_ERR_CUDA for the last launch
int sm_count();                     // SMs of the current device (cached)
int grid_for(const void* kernel, int block, size_t smem, int64_t work_blocks);

// Opt-in for dynamic shared memory: a launch gets 48 KB of shared memory
// (static and dynamic together) unless the kernel's attribute allows more,
// so the attribute is raised whenever the dynamic part alone exceeds 32 KB
// (the static shared memory of the kernels launched this way stays below
// 16 KB).
template <typename K>
inline int opt_in_smem(K kfn, size_t smem) {
  if (smem <= 32 * 1024) return TQ_OK;
  const cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return e == cudaSuccess ? TQ_OK : set_cuda_error(e);
}

inline bool valid_dtype(int d) { return d == TQ_F32 || d == TQ_F64; }
inline size_t dtype_size(int d) { return d == TQ_F64 ? 8 : 4; }

// Workspace layout shared by the reducing kernels: a 16-byte ticket word
// followed by `slots` compensated pairs (2 doubles each).
inline size_t reduce_ws_bytes(int64_t slots) { return 256 + (size_t)slots * 16; }

// ------------------------------------------------- compensated accumulation
// Neumaier's variant of Kahan summation: exact error term of each addition.
struct Acc {
  double s, c;
};
__device__ __forceinline__ void acc_add(Acc& a, double x) {
  double t = a.s + x;
  double e = (fabs(a.s) >= fabs(x)) ? ((a.s - t) + x) : ((x - t) + a.s);
  a.c += e;
  a.s = t;
}
__device__ __forceinline__ void acc_merge(Acc& a, const Acc& b) {
  acc_add(a, b.s);
  a.c += b.c;
}
__device__ __forceinline__ Acc acc_shfl_down(const Acc& a, int off) {
  Acc r;
  r.s = __shfl_down_sync(0xffffffffu, a.s, off);
  r.c = __shfl_down_sync(0xffffffffu, a.c, off);
  return r;
}
// Fixed-order reduction of one Acc per thread (blockDim.x <= BLOCK, whole
// warps); result valid in thread 0.  One warp combines the partials: lane l
// merges partials l, l + 32, ... in order, then the lanes in a shuffle tree.
// (Merging in every warp first ran five compensated merges on all 256
// threads: on GB300, where an FP64 warp instruction holds the FP64 unit for
// about 64 cycles, that cost more than the grid itself for a C1-sized
// fused launch.)
template <int BLOCK>
__device__ __forceinline__ Acc block_reduce(Acc a) {
  __shared__ Acc part[BLOCK];
  part[threadIdx.x] = a;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nt = min(BLOCK, (int)blockDim.x);
    Acc r = part[threadIdx.x];
    for (int i = threadIdx.x + 32; i < nt; i += 32) acc_merge(r, part[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc_merge(r, acc_shfl_down(r, off));
    a = r;
  }
  __syncthreads();
  return a;
}

// fp32 compensated strip accumulator (cheap on the FP32 pipe).
struct AccF {
  float s, c;
};
__device__ __forceinline__ void accf_add(AccF& a, float x) {
  float t = __fadd_rn(a.s, x);
  float e = (fabsf(a.s) >= fabsf(x)) ? __fadd_rn(__fsub_rn(a.s, t), x)
                                     : __fadd_rn(__fsub_rn(x, t), a.s);
  a.c = __fadd_rn(a.c, e);
  a.s = t;
}

// Double-float (two-float) accumulation on the FP32 pipe: the unevaluated
// sum hi + lo, |lo| <= ulp(hi) / 2, about 48 significant bits.  Additions
// use Knuth's TwoSum and Dekker's Fast2Sum for the renormalisation (the
// accurate variant: two TwoSums per addition, so cancellation between terms
// of either sign keeps the bound).  On GB300 an FP64 warp instruction
// occupies an SM sub-partition's FP64 unit for about 64 cycles; these
// operations keep long reductions off that unit.
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return F2{s, e};
}
__device__ __forceinline__ F2 fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return F2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  F2 s = two_sum(a.hi, b.hi);
  const F2 t = two_sum(a.lo, b.lo);
  s = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ F2 f2_add(F2 a, float b) {
  const F2 s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ F2 f2_shfl_down(F2 a, int off) {
  return F2{__shfl_down_sync(0xffffffffu, a.hi, off), __shfl_down_sync(0xffffffffu, a.lo, off)};
}
__device__ __forceinline__ F2 f2_shfl_up(F2 a, int off) {
  return F2{__shfl_up_sync(0xffffffffu, a.hi, off), __shfl_up_sync(0xffffffffu, a.lo, off)};
}
__device__ __forceinline__ double f2_value(F2 a) { return (double)a.hi + (double)a.lo; }
// Products (Dekker's TwoProduct through an FMA, then one renormalisation):
// about 48 significant bits, FP32 pipe only.
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ F2 f2_mul(F2 a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}
// A double split into a double-float (two conversions; once per set-up).
__device__ __forceinline__ F2 f2_from_double(double x) {
  const float hi = __double2float_rn(x);
  return F2{hi, __double2float_rn(x - (double)hi)};
}
// The double-float rounded to the nearest float.
__device__ __forceinline__ float f2_round(F2 a) { return __fadd_rn(a.hi, a.lo); }

// A double split into two floats by integer operations alone (no FP64
// instruction; on GB300 conversions also occupy the FP64 unit): hi takes the
// sign, the exponent and the leading 24 significant bits (truncated), lo the
// remaining 29 bits rounded to 23, so |x - (hi + lo)| <= 2^-47 |x|, without
// bias.  lo comes from a float whose exponent is known, 2^(e-1046) + q
// 2^(e-1069) with q the rounded top 23 of the 29 bits, minus 2^(e-1046)
// (exact).  Branch-free.  Only 2^-40 <= |x| < 2^40 is split, so that
// weighted products and long sums of such values stay far inside the float
// range; otherwise hi = lo = 0, and ok is false unless x is a zero: other
// values (small, large, subnormal, infinite, NaN) are the caller's to
// handle in fp64.
struct F2Split {
  F2 v;
  bool ok;
};
__device__ __forceinline__ F2Split f2_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t bh = (uint32_t)(b >> 32), bl = (uint32_t)b;
  const uint32_t em = bh & 0x7ff00000u;  // biased binary exponent e, << 20
  const uint32_t sgn = bh & 0x80000000u;
  F2Split r;
  const bool in = em - (983u << 20) <= (79u << 20) + 0xfffffu;  // 983 <= e <= 1062
  // bits 30..23: the low 8 bits of e, 22..0: fraction bits 51..29; the
  // float exponent e - 896 is those 8 bits with the top one flipped
  const uint32_t fs = __funnelshift_l(bl, bh, 3);
  const float hi = __uint_as_float(((fs ^ 0x40000000u) & 0x7fffffffu) | sgn);
  const uint32_t ex = em * 8u - (919u << 23);
  const uint32_t q = ((bl & 0x1fffffffu) + 32u) >> 6;  // a carry into the exponent stays exact
  const float lo = __fsub_rn(__uint_as_float(ex + q), __uint_as_float(ex));
  r.v.hi = in ? hi : 0.f;
  r.v.lo = in ? __uint_as_float(__float_as_uint(lo) | sgn) : 0.f;
  r.ok = in || ((bh & 0x7fffffffu) | bl) == 0u;
  return r;
}

// "Last CTA finishes" pattern: every CTA writes its partial, fences, takes a
// ticket; the CTA that draws the last ticket reduces all partials in index
// order (deterministic) and resets the ticket for the next launch.  No CTA
// waits on another, so nothing can spin.
// `count` CTAs take part (a kernel whose CTAs play several roles counts
// each role's CTAs on its own ticket).
__device__ __forceinline__ bool last_block_of(unsigned* ticket, unsigned count) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(ticket, 1u);
    is_last = (t == count - 1);
  }
  __syncthreads();
  return is_last;
}
__device__ __forceinline__ bool last_block_arrives(unsigned* ticket) {
  return last_block_of(ticket, gridDim.x * gridDim.y * gridDim.z);
}

// ------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11: 10 rounds of the 4x32 bijection with multipliers 0xD2511F53 /
// 0xCD9E8D57 and Weyl key increments 0x9E3779B9 / 0xBB67AE85.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
    const uint32_t lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}
__device__ __forceinline__ uint4 philox_block(uint64_t seed, uint64_t stream_id,
                                              uint64_t block) {
  return philox4x32_10(make_uint4((uint32_t)block, (uint32_t)(block >> 32),
                                  (uint32_t)stream_id, (uint32_t)(stream_id >> 32)),
                       make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}
__device__ __forceinline__ uint32_t lane_of(const uint4& r, int l) {
  return l == 0 ? r.x : l == 1 ? r.y : l == 2 ? r.z : r.w;
}
__device__ __forceinline__ float u32_to_unit_f(uint32_t r) {
  return (float)(r >> 8) * 5.9604644775390625e-08f;  // 2^-24
}
__device__ __forceinline__ double u64_to_unit_d(uint32_t lo, uint32_t hi) {
  const uint64_t x = (((uint64_t)hi << 32) | lo) >> 11;
  return (double)x * 1.1102230246251565e-16;  // 2^-53
}
// Uniform number of flat element e of a request starting at block `offset`.
template <typename T>
struct Uniform;
template <>
struct Uniform<float> {
  static constexpr int per_block = 4;
  __device__ static float at(uint64_t seed, uint64_t sid, uint64_t offset, uint64_t e) {
    const uint4 r = philox_block(seed, sid, offset + (e >> 2));
    return u32_to_unit_f(lane_of(r, (int)(e & 3)));
  }
  __device__ static float from(const uint4& r, int lane) {
    return u32_to_unit_f(lane_of(r, lane));
  }
};
template <>
struct Uniform<double> {
  static constexpr int per_block = 2;
  __device__ static double at(uint64_t seed, uint64_t sid, uint64_t offset, uint64_t e) {
    const uint4 r = philox_block(seed, sid, offset + (e >> 1));
    return (e & 1) ? u64_to_unit_d(r.z, r.w) : u64_to_unit_d(r.x, r.y);
  }
  __device__ static double from(const uint4& r, int lane) {
    return lane ? u64_to_unit_d(r.z, r.w) : u64_to_unit_d(r.x, r.y);
  }
};

// --------------------------------------------- division by an invariant
// Unsigned 32-bit division by a run-time constant d >= 1 with one multiply-
// high, the round-up method of Granlund & Montgomery, "Division by invariant
// integers using multiplication" (PLDI 1994), Fig. 4.1:
//   l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
//   q = (t + ((n - t) >> min(l,1))) >> max(l-1,0), t = mulhi(m, n).
struct FastDiv {
  uint32_t d, m, s1, s2;
};
__host__ __device__ inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  uint32_t l = 0;
  while (l < 32 && (uint64_t(1) << l) < d) ++l;
  f.d = d;
  f.m = (uint32_t)(((uint64_t(1) << 32) * ((uint64_t(1) << l) - d)) / d + 1);
  f.s1 = l < 1 ? l : 1;
  f.s2 = l > 1 ? l - 1 : 0;
  return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  const uint32_t t = __umulhi(f.m, n);
  return (t + ((n - t) >> f.s1)) >> f.s2;
}

// ------------------------------------------------------------- grid nodes
// torch's CPU linspace, which IntegrationGrid uses through
// _linspace_with_grads (utils.py:24-58): step = (b-a)/(n-1) in the working
// type, the first half of the nodes from a forwards, the rest from b
// backwards, each a single rounding of step*i +- endpoint.
template <typename T>
__device__ __forceinline__ T linspace_node(T a, T b, T step, int64_t n, int64_t i) {
  if (i < n / 2) return fma(step, (T)i, a);
  return fma(-step, (T)(n - 1 - i), b);
}

// 1-D composite weights without the h factor, normalised so that the
// weight of node i is h * nc_coef(rule, i, n) (trapezoid.py:35,
// simpson.py:73-80, boole.py:154-163 collapse to these coefficients).
__device__ __forceinline__ double nc_coef(int rule, int64_t i, int64_t n) {
  if (rule == TQ_RULE_TRAPEZOID) return (i == 0 || i == n - 1) ? 0.5 : 1.0;
  if (rule == TQ_RULE_SIMPSON) {
    if (i == 0 || i == n - 1) return 1.0 / 3.0;
    return (i & 1) ? 4.0 / 3.0 : 2.0 / 3.0;
  }
  // Boole: h/22.5 * (7, 32, 12, 32, 14, 32, 12, 32, ..., 7)
  if (i == 0 || i == n - 1) return 7.0 / 22.5;
  const int64_t m = i & 3;
  if (m == 1 || m == 3) return 32.0 / 22.5;
  if (m == 2) return 12.0 / 22.5;
  return 14.0 / 22.5;
}

// ------------------------------------------------------- integrand families
template <typename T>
struct Family {
  int id, dim;
  T c, b;
  T a[kMaxDim];
  T u[kMaxDim];
};
template <typename T>
__device__ __forceinline__ void load_family(Family<T>& f, int id, int dim,
                                            const double* __restrict__ p) {
  f.id = id;
  f.dim = dim;
  f.c = (T)p[0];
  f.b = (T)p[1];
#pragma unroll
  for (int k = 0; k < kMaxDim; ++k) {
    f.a[k] = k < dim ? (T)p[2 + k] : T(0);
    f.u[k] = (k < dim && id == TQ_FN_GAUSSIAN) ? (T)p[2 + dim + k] : T(0);
  }
}
// g_k(x_k): the per-dimension term of the separable sum.
template <int FAM, typename T>
__device__ __forceinline__ T fam_term(const Family<T>& f, int k, T x) {
  if (FAM == TQ_FN_GAUSSIAN) {
    const T d = x - f.u[k];
    return f.a[k] * (d * d);
  } else if (FAM == TQ_FN_SUM_SIN) {
    return sin(f.a[k] * x);
  } else {
    return f.a[k] * x;
  }
}
// F(s): the outer function of the separable sum.
template <int FAM, typename T>
__device__ __forceinline__ T fam_outer(const Family<T>& f, T s) {
  if (FAM == TQ_FN_EXP_SUM) return f.c * exp(s + f.b);
  if (FAM == TQ_FN_GAUSSIAN) return f.c * exp(-s);
  if (FAM == TQ_FN_OSCILLATORY) return f.c * cos((T)(2.0 * CUDART_PI) * f.b + s);
  return f.c * s;  // TQ_FN_SUM_SIN
}

}  // namespace tq

// Dispatch helpers: expand a runtime family id into a template argument.
#define TQ_DISPATCH_FAMILY(fam, FAMC, ...)                    \
  switch (fam) {                                              \
    case TQ_FN_EXP_SUM: {                                     \
      constexpr int FAMC = TQ_FN_EXP_SUM;                     \
      __VA_ARGS__;                                            \
    } break;                                                  \
    case TQ_FN_GAUSSIAN: {                                    \
      constexpr int FAMC = TQ_FN_GAUSSIAN;                    \
      __VA_ARGS__;                                            \
    } break;                                                  \
    case TQ_FN_OSCILLATORY: {                                 \
      constexpr int FAMC = TQ_FN_OSCILLATORY;                 \
      __VA_ARGS__;                                            \
    } break;                                                  \
    case TQ_FN_SUM_SIN: {                                     \
      constexpr int FAMC = TQ_FN_SUM_SIN;                     \
      __VA_ARGS__;                                            \
    } break;                                                  \
    default:                                                  \
      return TQ_ERR_FAMILY;                                   \
  }
