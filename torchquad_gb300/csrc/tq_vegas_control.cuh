// Control of a VEGAS run on the device: the per-call inputs of a run
// (begin_run_body) and the reference's abort test after every fifth
// iteration (abort_body), shared by the per-launch kernels (tq_vegas_loop.cu)
// and the kernels that advance many states per launch (tq_vegas_batch.cu).
//
// Reference (torchquad v0.5.0): vegas.py:100-209 (VEGAS.integrate and
// _check_abort_conditions), :318-362 (_get_result, _get_error, _get_chisq).
#pragma once

#include <math.h>
#include <string.h>

#include "tq_common.cuh"

namespace tq {

enum : int {
  kCtlNevals = 0,
  kCtlSlot = 1,
  kCtlNormalize = 2,
  kCtlSeed = 3,
  kCtlStream = 4,
  kCtlN = 5,
  kCtlNInc = 6,
  kCtlMaxIt = 7,
  kCtlEpsRel = 8,
  kCtlEpsAbs = 9,
  kCtlWarm = 10,
  kCtlIt = 11,
  kCtlStop = 12,
  kCtlEvals = 13,
};

struct RunArgs {
  tq_vegas_run run;
  int64_t* control;
  uint64_t* rng_offset;
  double* params_dev;
  void* domain;  // the state's [dim][2] domain buffer
  int dtype;
};

// The run inputs r into a state's control block, RNG offset, parameter
// vector and domain buffer (one thread).  At most max_params parameters and
// max_domain domain values are copied (the state's 2 + 2 dim and 2 dim: a
// run record read from device memory is bounded by its state, not trusted).
static __device__ void begin_run_from(const tq_vegas_run& r, int64_t* c, uint64_t* rng_offset,
                                      double* params_dev, void* domain, int dtype,
                                      int max_params = 2 + 2 * TQ_MAX_DIM, int max_domain = 2 * TQ_MAX_DIM) {
  c[kCtlNevals] = r.nevals_exp;
  c[kCtlSeed] = (int64_t)r.seed;
  c[kCtlStream] = (int64_t)r.stream_id;
  c[kCtlN] = r.N;
  c[kCtlNInc] = r.N_increment;
  c[kCtlMaxIt] = r.max_iterations;
  c[kCtlEpsRel] = __double_as_longlong(r.eps_rel);
  c[kCtlEpsAbs] = __double_as_longlong(r.eps_abs);
  c[kCtlWarm] = r.warm_evals;
  c[kCtlIt] = 0;
  c[kCtlStop] = 0;
  c[kCtlEvals] = r.warm_evals;
  *rng_offset = r.rng_offset;
  const int n_params = r.n_params < 0 ? 0 : (r.n_params > max_params ? max_params : r.n_params);
  const int n_domain = r.n_domain == max_domain ? max_domain : 0;  // the whole domain or none
  for (int i = 0; i < n_params; ++i) params_dev[i] = r.params[i];
  for (int i = 0; i < n_domain; ++i) {
    if (dtype == TQ_F64)
      ((double*)domain)[i] = r.domain[i];
    else
      ((float*)domain)[i] = __double2float_rn(r.domain[i]);
  }
}

static __device__ void begin_run_body(const RunArgs& a) {
  // the host checked n_params and n_domain (tq_vegas_begin_run)
  begin_run_from(a.run, a.control, a.rng_offset, a.params_dev, a.domain, a.dtype, a.run.n_params,
                 a.run.n_domain);
}

// Arithmetic of the abort test in the state's dtype, each operation rounded
// once to nearest (the reference does it on 0-d tensors of that dtype); the
// quotients give IEEE results for x / 0 (+-inf or NaN), as tensors do.
static __device__ __forceinline__ float a_add(float x, float y) { return __fadd_rn(x, y); }
static __device__ __forceinline__ double a_add(double x, double y) { return __dadd_rn(x, y); }
static __device__ __forceinline__ float a_sub(float x, float y) { return __fsub_rn(x, y); }
static __device__ __forceinline__ double a_sub(double x, double y) { return __dsub_rn(x, y); }
static __device__ __forceinline__ float a_mul(float x, float y) { return __fmul_rn(x, y); }
static __device__ __forceinline__ double a_mul(double x, double y) { return __dmul_rn(x, y); }
static __device__ __forceinline__ float a_div(float x, float y) { return __fdiv_rn(x, y); }
static __device__ __forceinline__ double a_div(double x, double y) { return __ddiv_rn(x, y); }
static __device__ __forceinline__ float a_sqrt(float x) { return __fsqrt_rn(x); }
static __device__ __forceinline__ double a_sqrt(double x) { return __dsqrt_rn(x); }
static __device__ __forceinline__ float a_cast(double x, float) { return __double2float_rn(x); }
static __device__ __forceinline__ double a_cast(double x, double) { return x; }

// _check_abort_conditions for the block that just ended, in the host code's
// operation order (every sum left to right from zero), on one warp, in the
// state's dtype T: lane i < 5 holds result r_i and variance s_i of the
// block's i-th iteration.  The quotients of the rows are taken by their own
// lanes at once (the same operations as one thread would do); the sums and
// the decision are taken by every lane alike.  Python scalars meet the
// tensors as T (eps_rel, eps_abs, eps_rel + 1e-8, 5.0 and _starting_N are
// rounded to T first, as torch does with a scalar operand).  Returns the
// stop reason (0: go on; 5 / 6: int() of an infinite / NaN value, where the
// reference raises) and updates *sN (VEGAS._starting_N).
template <typename T>
__device__ int abort_decision_warp(double r_in, double s_in, int64_t it, int64_t evals, int64_t N,
                                   int64_t n_inc, int64_t max_it, double eps_rel_d,
                                   double eps_abs_d, int64_t* sN) {
  const int lane = threadIdx.x & 31;
  const bool row = lane < 5;
  const T zero = (T)0, one = (T)1, five = (T)5;
  const T r_mine = a_cast(r_in, zero), s_mine = a_cast(s_in, zero);
  const unsigned zeros = __ballot_sync(0xffffffffu, row && s_mine == zero);
  const T q_mine = row ? a_div(r_mine, s_mine) : zero;  // r_i / s_i
  const T inv_mine = row ? a_div(one, s_mine) : zero;   // 1 / s_i
  T r[5], s[5], q[5], inv[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    r[i] = __shfl_sync(0xffffffffu, r_mine, i);
    s[i] = __shfl_sync(0xffffffffu, s_mine, i);
    q[i] = __shfl_sync(0xffffffffu, q_mine, i);
    inv[i] = __shfl_sync(0xffffffffu, inv_mine, i);
  }
  // _get_result (EQ 30)
  T res;
  if (zeros) {
    T t = zero;
    for (int i = 0; i < 5; ++i) t = a_add(t, r[i]);
    res = a_div(t, five);
  } else {
    T num = zero, den = zero;
    for (int i = 0; i < 5; ++i) {
      num = a_add(num, q[i]);
      den = a_add(den, inv[i]);
    }
    res = a_div(num, den);
  }
  const T res_abs = res < zero ? -res : res;
  // _get_error (EQ 31)
  T isum = zero;
  for (int i = 0; i < 5; ++i)
    if (s[i] != zero) isum = a_add(isum, inv[i]);
  const T err = isum == zero ? s[0] : a_div(one, a_sqrt(isum));
  // _get_chisq (EQ 32): each row's term on its lane, summed in row order
  const bool use = row && r_mine != res;
  T term = zero;
  if (use) {
    const T d = a_sub(r_mine, res);
    term = a_div(a_mul(d, d), s_mine);
  }
  const unsigned used = __ballot_sync(0xffffffffu, use);
  T chi2 = zero;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const T t = __shfl_sync(0xffffffffu, term, i);
    if (used >> i & 1u) chi2 = a_add(chi2, t);
  }
  const T eps_rel = a_cast(eps_rel_d, zero), eps_abs = a_cast(eps_abs_d, zero);
  const T qc = a_div(chi2, five);
  if ((err <= a_mul(eps_rel, res_abs) || err <= eps_abs) && qc < one) return 1;
  if (qc < one) {
    if (res_abs == zero) {
      *sN += n_inc;
    } else {
      const T acc = a_div(err, res_abs);
      const T x = a_mul(a_cast((double)*sN, zero), a_sqrt(a_div(acc, a_cast(eps_rel_d + 1e-8, zero))));
      // int(): truncation toward zero; the reference raises for a value
      // that is not finite
      if (isnan(x)) return 6;
      if (isinf(x)) return 5;
      const int64_t t = __double2ll_rz((double)x);
      *sN = min(*sN + n_inc, t);
    }
  } else if (qc > one) {
    *sN += n_inc;
  }
  if (evals + *sN * 5 > N) return 2;
  if (it + 5 > max_it) return 3;
  return 0;
}

struct AbortArgs {
  int64_t* control;
  int dtype;
  const double* stats;
  int64_t n_stat_slots;
  cudaGraphConditionalHandle handle;
  int use_handle;
};

// One warp: the statistics rows are loaded by all lanes at once (the
// evaluation count is an exact integer sum); lane 0 writes the outcome.
// One warp (lanes 0..31 of the calling CTA).
static __device__ void abort_body(const AbortArgs& a) {
  int64_t* c = a.control;
  const int lane = threadIdx.x;
  const int64_t slot = c[kCtlSlot];  // rows [slot - 5, slot) hold this block
  const bool ok = slot >= 5 && slot <= a.n_stat_slots;
  int64_t evals = 0;  // _nr_of_fevals: the warm-up plus the points of every iteration so far
  double r_mine = 0.0, s_mine = 0.0;
  if (ok) {
    for (int64_t i = lane; i < slot; i += 32) evals += (int64_t)a.stats[4 * i + 2];
    if (lane < 5) {
      r_mine = a.stats[4 * (slot - 5 + lane)];
      s_mine = a.stats[4 * (slot - 5 + lane) + 1];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
  const int64_t it = c[kCtlIt] + 5;
  int stop = 4;  // the statistics slots ran out: nothing valid to test
  int64_t sN = c[kCtlNevals];
  evals += c[kCtlWarm];
  if (ok) {
    const double er = __longlong_as_double(c[kCtlEpsRel]), ea = __longlong_as_double(c[kCtlEpsAbs]);
    stop = a.dtype == TQ_F32 ? abort_decision_warp<float>(r_mine, s_mine, it, evals, c[kCtlN], c[kCtlNInc],
                                                          c[kCtlMaxIt], er, ea, &sN)
                             : abort_decision_warp<double>(r_mine, s_mine, it, evals, c[kCtlN],
                                                           c[kCtlNInc], c[kCtlMaxIt], er, ea, &sN);
  }
  if (lane != 0) return;
  if (ok) {
    c[kCtlEvals] = evals;
    c[kCtlNevals] = sN;
  }
  c[kCtlIt] = it;
  c[kCtlStop] = stop;
  if (a.use_handle) cudaGraphSetConditional(a.handle, stop == 0 ? 1u : 0u);
}

}  // namespace tq
