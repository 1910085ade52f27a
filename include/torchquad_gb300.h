/*
 * torchquad_gb300 — C ABI of the GB300 (sm_103a) integration kernels.
 *
 * Every entry point:
 *   - takes plain device pointers, sizes and a cudaStream_t passed as void*;
 *   - never allocates device memory except where a comment says so (the
 *     caller passes every buffer, scratch included, sized by the matching
 *     *_workspace_size() query);
 *   - never throws and never synchronises the stream; it returns an int
 *     status (TQ_OK or a negative TQ_ERR_* code, see tq_status_string()).
 *
 * Arrays are row-major.  "dtype" selects the arithmetic type of points,
 * integrand values and integration domain: TQ_F32 or TQ_F64.  Sums are
 * accumulated in fp64 with compensated (Neumaier/Kahan) summation whatever
 * the dtype.
 *
 * Each declaration names the reference torchquad (v0.5.0) function it
 * replaces as file:line within the reference project.
 */
#ifndef TORCHQUAD_GB300_H
#define TORCHQUAD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
  TQ_OK = 0,
  TQ_ERR_ARG = -1,         /* null pointer / inconsistent sizes            */
  TQ_ERR_DIM = -2,         /* dim < 1 or dim > TQ_MAX_DIM on a fused path  */
  TQ_ERR_RULE = -3,        /* unknown rule or n invalid for the rule       */
  TQ_ERR_FAMILY = -4,      /* unknown built-in integrand family            */
  TQ_ERR_TOO_LARGE = -5,   /* point count overflows the index arithmetic   */
  TQ_ERR_WORKSPACE = -6,   /* workspace smaller than *_workspace_size()    */
  TQ_ERR_CUDA = -7,        /* a CUDA runtime call failed (tq_last_cuda_error) */
  TQ_ERR_DTYPE = -8,       /* unknown dtype code                           */
  TQ_ERR_TIMEOUT = -9,     /* a bounded device-side wait gave up           */
  TQ_ERR_SCRATCH = -10     /* needs more than the static scratch of
                            * tq_grid_fused_noalloc holds                  */
};

enum { TQ_F32 = 0, TQ_F64 = 1 };

/* Quadrature rules (reference: trapezoid.py:27-37, simpson.py:29-46,
 * boole.py:29-48, gaussian.py:131-144; TQ_RULE_MC is the plain mean of
 * monte_carlo.py:60-82). */
enum {
  TQ_RULE_TRAPEZOID = 0,
  TQ_RULE_SIMPSON = 1,
  TQ_RULE_BOOLE = 2,
  TQ_RULE_GAUSS = 3,
  TQ_RULE_MC = 4
};

/* Built-in fused integrand families.  Every family has the separable-sum
 * form f(x) = F(sum_k g_k(x_k)); params is a device fp64 array
 *   params[0] = c, params[1] = b, params[2 .. 2+dim) = a_k,
 *   params[2+dim .. 2+2*dim) = u_k   (only TQ_FN_GAUSSIAN reads u_k)
 *
 *   TQ_FN_EXP_SUM      f = c * exp(sum_k a_k x_k + b)
 *   TQ_FN_GAUSSIAN     f = c * exp(-sum_k a_k (x_k - u_k)^2)
 *   TQ_FN_OSCILLATORY  f = c * cos(2*pi*b + sum_k a_k x_k)
 *   TQ_FN_SUM_SIN      f = c * sum_k sin(a_k x_k)
 */
enum {
  TQ_FN_PER_DESC = -1, /* batched calls: each descriptor names its own family */
  TQ_FN_EXP_SUM = 1,
  TQ_FN_GAUSSIAN = 2,
  TQ_FN_OSCILLATORY = 3,
  TQ_FN_SUM_SIN = 4
};

#define TQ_MAX_DIM 16

/* ---- library ------------------------------------------------------------- */
const char* tq_status_string(int status);
/* The cudaError_t of the last TQ_ERR_CUDA on the calling thread. */
int tq_last_cuda_error(void);
/* Number of SMs and resident CTAs the grids are sized with (device current). */
int tq_device_sm_count(void);

/* ---- grid rules: fused (node generation + integrand + weighted sum) ------ */

/* Workspace bytes needed by tq_grid_fused for this problem. */
size_t tq_grid_fused_workspace_size(int rule, int dim, int64_t n_per_dim);

/* Tensor-product rule over n_per_dim^dim nodes with a built-in integrand,
 * written to out[0] (dtype out_dtype) and, if out64 != NULL, to out64[0].
 * Replaces GridIntegrator.integrate (grid_integrator.py:32-55) for the
 * Trapezoid/Simpson/Boole/GaussLegendre subclasses: IntegrationGrid
 * (integration_grid.py:28-103) + evaluate_integrand (base_integrator.py:43-91)
 * + calculate_result/_apply_composite_rule (grid_integrator.py:57-91).
 * domain: device [dim][2] of dtype; gl_nodes/gl_weights: device fp64 [n]
 * Gauss-Legendre roots/weights on [-1,1] (only for TQ_RULE_GAUSS, whose
 * nodes are computed in fp64 as in gaussian.py:159-162). */
int tq_grid_fused(int dtype, int rule, int dim, int64_t n_per_dim,
                  const void* domain, const double* gl_nodes,
                  const double* gl_weights, int family, const double* params,
                  void* out, int out_dtype, double* out64,
                  void* workspace, size_t workspace_bytes, void* stream);

/* tq_grid_fused without a workspace argument, for callers that cannot
 * allocate device memory when they call (no counterpart in the reference).
 * Scratch is a static device array of 256 B + 4096 CTA partials (64 KiB),
 * enough for grids of up to 8 CTAs per SM on GPUs of up to 512 SMs; a
 * request needing more returns TQ_ERR_SCRATCH.  The first call on a device
 * looks the array's address up (cudaGetSymbolAddress); make that first call
 * before any stream capture.  Every call shares the one array, so calls that
 * overlap on the GPU (other streams, other host threads) race: serialise
 * them.  Allocates nothing. */
int tq_grid_fused_noalloc(int dtype, int rule, int dim, int64_t n_per_dim,
                          const void* domain, const double* gl_nodes,
                          const double* gl_weights, int family, const double* params,
                          void* out, int out_dtype, double* out64, void* stream);

/* ---- batched grid rules ---------------------------------------------------- */

/* Descriptor of one integral of a batch (56 bytes, int64-aligned). */
typedef struct tq_batch_desc {
  int32_t rule, dim;   /* TQ_RULE_TRAPEZOID..TQ_RULE_GAUSS, 1..TQ_MAX_DIM        */
  int64_t n, total;    /* points per dimension, n^dim                          */
  int64_t par_off;     /* offset of the integral's 2+2*dim parameters in params */
  int64_t dom_off;     /* offset of its [dim][2] domain in domains (dtype)      */
  int64_t gl_off;      /* offset of its n Gauss roots/weights (fp64)           */
  int32_t family;      /* TQ_FN_* (read when the call's family is TQ_FN_PER_DESC) */
  int32_t pad;
} tq_batch_desc;

/* Many tensor-product integrals of built-in families in one persistent
 * launch (no counterpart in the reference, whose batch is a loop of
 * GridIntegrator.integrate, grid_integrator.py:32-55).  family is one
 * TQ_FN_* for every integral, or TQ_FN_PER_DESC to take each descriptor's
 * (families mixed in one launch).  Integral i is cut
 * into ceil(total_i / tile_points) tiles; tile_start[n_integrals+1] is the
 * exclusive prefix of the tile counts (tile_start[n_integrals] = n_tiles).
 * block (128|256), strip (4|16 nodes per thread) and grid_blocks (0: 8 per
 * SM) are the tunable launch shape.  out[i] (out_dtype) receives integral
 * i; workspace >= n_tiles * 16 bytes. */
int tq_batch_grid(int dtype, int64_t n_integrals, const void* descs, const int64_t* tile_start,
                  int64_t n_tiles, int64_t tile_points, const double* params,
                  const void* domains, const double* gl_nodes, const double* gl_weights,
                  int family, int block, int strip, int grid_blocks, void* out, int out_dtype,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Descriptor of one Monte Carlo chunk of a batch (56 bytes). */
typedef struct tq_mc_desc {
  int32_t dim, family;   /* family: TQ_FN_* (read when the call's is TQ_FN_PER_DESC) */
  int64_t first, count;  /* point range [first, first+count) of the stream */
  uint64_t seed, stream_id;
  int64_t par_off, dom_off;
} tq_mc_desc;

/* One chunk of each of many Monte Carlo integrations of built-in families
 * (family: one TQ_FN_* for all, or TQ_FN_PER_DESC for each descriptor's)
 * (no counterpart in the reference; its MonteCarlo.integrate,
 * monte_carlo.py:20-106, does one integral per call).  Request r evaluates
 * points [first, first+count) of its Philox stream (point p uses elements
 * p*dim .. p*dim+dim-1 of tq_uniform's layout at block offset 0) with
 * x = u * (b - a) + a, and adds sum f, sum f^2 to acc[r][0..1] and
 * acc[r][2..3] (compensated pairs).  tile_start[n_requests+1] is the prefix
 * of ceil(count / tile_points); workspace >= n_tiles * 32 bytes. */
int tq_batch_mc(int dtype, int64_t n_requests, const void* descs, const int64_t* tile_start,
                int64_t n_tiles, int64_t tile_points, const double* params, const void* domains,
                int family, double* acc, void* workspace, size_t workspace_bytes, void* stream);

/* ---- grid rules: adjoint --------------------------------------------------- */

size_t tq_grid_adjoint_workspace_size(int dim, int64_t total_points);

/* Value and gradient of the fused tensor-product rule (dim <= 8):
 * out_value[0] = I, out_grad_domain[k][0|1] = dI/da_k | dI/db_k,
 * out_grad_params[i] = dI/dparams[i] (same layout as params: c, b, a_k, u_k).
 * fp64 grids of the exponential and oscillatory families with a node table
 * (dim >= 2, at most 256 nodes per dimension) sum their node terms as
 * double-floats (about 2^-47 per operation), the rest in fp64.
 * Replaces torch autograd through the reference's materialised grid
 * (integration_grid.py:74-88, utils.py:36-52, gaussian.py:81-84,159-162);
 * the domain gradient is that of nodes a + t (b - a) with weights
 * proportional to prod (b - a), as in those code paths. */
int tq_grid_adjoint(int dtype, int rule, int dim, int64_t n_per_dim, const void* domain,
                    const double* gl_nodes, const double* gl_weights, int family,
                    const double* params, double* out_value, double* out_grad_domain,
                    double* out_grad_params, void* workspace, size_t workspace_bytes,
                    void* stream);

/* Workspace bytes of tq_batch_grid_adjoint: n_tiles rows of 2 + 4*max_dim
 * fp64 partial sums. */
size_t tq_batch_grid_adjoint_workspace_size(int64_t n_tiles, int max_dim);

/* Value and gradient of many tensor-product integrals of built-in families
 * (dims <= 8) in one persistent launch, the batched form of tq_grid_adjoint
 * (the reference differentiates each integral separately through torch
 * autograd over its materialised grid: integration_grid.py:74-88,
 * utils.py:36-52, gaussian.py:81-84).  descs / tile_start / params /
 * domains / gl_* as for tq_batch_grid (family per descriptor unless family
 * >= 0); max_dim: the largest dim of the batch.  Writes, per integral i,
 * out_value[i] (fp64), out_grad_domain at the integral's dom_off ([dim][2],
 * fp64: dI/da_k, dI/db_k) and out_grad_params at its par_off (fp64, the
 * layout of params).  Tiles are summed in tile order: the results do not
 * depend on the other integrals of the batch. */
int tq_batch_grid_adjoint(int dtype, int64_t n_integrals, const void* descs,
                          const int64_t* tile_start, int64_t n_tiles, int64_t tile_points,
                          const double* params, const void* domains, const double* gl_nodes,
                          const double* gl_weights, int family, int max_dim, double* out_value,
                          double* out_grad_domain, double* out_grad_params, void* workspace,
                          size_t workspace_bytes, void* stream);

/* ---- grid rules: materialised path for arbitrary integrands -------------- */

/* Writes points[count][dim] (dtype; fp64 for TQ_RULE_GAUSS) for the flat
 * node indices [start, start+count) of the tensor-product grid, last
 * dimension fastest, exactly as IntegrationGrid builds them
 * (integration_grid.py:95-99 meshgrid(indexing="ij") + stack). */
int tq_grid_points(int dtype, int rule, int dim, int64_t n_per_dim,
                   const void* domain, const double* gl_nodes,
                   int64_t start, int64_t count, void* points, void* stream);

/* Writes the tensor-product quadrature weight of each node in
 * [start, start+count) to weights[count] (fp64).  Used by the backward pass
 * of the differentiable materialised path (d result / d f_i). */
int tq_grid_weights(int dtype, int rule, int dim, int64_t n_per_dim,
                    const void* domain, const double* gl_weights,
                    int64_t start, int64_t count, double* weights, void* stream);

size_t tq_weighted_sum_workspace_size(int64_t count, int64_t n_values);

/* acc[2*s], acc[2*s+1] (a compensated fp64 running sum, s < n_values) +=
 * sum_i w_i * f[i][s] over the nodes [start, start+count) of the grid;
 * f is [count][n_values] of f_dtype (complex integrands are passed as their
 * real view).  For TQ_RULE_MC w_i = 1.  One fp64 component of a grid rule
 * with 32 <= n_per_dim <= 2048 and (dim - 1) * n_per_dim <= 2048 is summed
 * as double-floats within each CTA (each term to about 2^-46 relative, the
 * sum's error bound of the order of an fp64 pairwise sum's).  Replaces the weight multiply of
 * base_integrator.py:77-89 and the per-dimension collapse of
 * grid_integrator.py:57-91 / the sum of monte_carlo.py:77. */
int tq_weighted_sum(int dtype, int rule, int dim, int64_t n_per_dim,
                    const void* domain, const double* gl_weights,
                    int64_t start, int64_t count, const void* f, int f_dtype,
                    int64_t n_values, double* acc, void* workspace,
                    size_t workspace_bytes, void* stream);

/* out[s] = (out_dtype)(scale * (acc[2s] + acc[2s+1])) where scale is 1 for
 * grid rules and prod_k(b_k - a_k) / n_points (computed in dtype, as
 * monte_carlo.py:72-77) for TQ_RULE_MC. */
int tq_finalize_sum(int dtype, int rule, int dim, const void* domain,
                    int64_t n_points, const double* acc, int64_t n_values,
                    void* out, int out_dtype, void* stream);

/* ---- random numbers ------------------------------------------------------ */

/* Counter-based Philox4x32-10 (Salmon et al., SC'11).  Element e of a
 * request with block offset `offset` is drawn from counter
 * {lo(offset+e/4), hi(offset+e/4), lo(stream_id), hi(stream_id)} lane e%4 for
 * fp32 (u = (r >> 8) * 2^-24) and from lanes 2(e%2), 2(e%2)+1 of block
 * offset+e/2 for fp64 (u = ((hi<<32|lo) >> 11) * 2^-53), key = seed.
 * All values lie in [0, 1).  A request of numel values consumes
 * ceil(numel/4) (fp32) or ceil(numel/2) (fp64) blocks.
 * Replaces RNG.uniform (rng.py:120-125, torch.rand). */
int tq_uniform(int dtype, uint64_t seed, uint64_t stream_id, uint64_t offset,
               int64_t numel, void* out, void* stream);

/* ---- Monte Carlo: fused ------------------------------------------------- */

size_t tq_mc_fused_workspace_size(int dim, int64_t n_points);

/* MonteCarlo.integrate (monte_carlo.py:20-106) for a built-in integrand:
 * x = u * (b - a) + a with u from tq_uniform(seed, stream_id, offset) over
 * [n_points][dim], result = prod(b - a) * sum f(x) / n_points -> out[0]. */
int tq_mc_fused(int dtype, int dim, int64_t n_points, const void* domain,
                int family, const double* params, uint64_t seed,
                uint64_t stream_id, uint64_t offset, void* out, double* out64,
                void* workspace, size_t workspace_bytes, void* stream);

/* ---- VEGAS+ (vegas.py, vegas_map.py, vegas_stratification.py) ---------- */

/* Device state of one VEGAS integration.  All arrays are caller-owned
 * device memory; "dtype" arrays use the state's dtype.  The adaptive map
 * lives on the unit cube [0,1]^dim; `domain` maps it onto the integration
 * domain as vegas.py:105-112 does. */
typedef struct tq_vegas_state {
  int32_t dim;          /* d, 1..TQ_MAX_DIM                                    */
  int32_t dtype;        /* TQ_F32 / TQ_F64                                     */
  int64_t n_bins;       /* B, map intervals per dimension (vegas.py:117)       */
  int64_t n_strat;      /* stratification steps per dimension                 */
  int64_t n_cubes;      /* n_strat^dim                                         */
  void* x_edges;        /* [d][B+1] dtype    VEGASMap.x_edges                  */
  void* dx_edges;       /* [d][B]   dtype    VEGASMap.dx_edges                 */
  double* weights;      /* [d][B]   sum of (f*jac)^2 per interval (fp64)       */
  int64_t* counts;      /* [d][B]   samples per interval                       */
  void* dh;             /* [n_cubes] dtype   VEGASStratification.dh            */
  double* jf;           /* [n_cubes] sum of f*jac per cube (fp64)              */
  double* jf2;          /* [n_cubes] sum of (f*jac)^2 per cube (fp64)          */
  int64_t* neval;       /* [n_cubes] evaluations per cube                     */
  int64_t* cube_start;  /* [n_cubes+1] exclusive prefix of neval; last = total */
  uint64_t* rng_offset; /* [1] Philox block offset; the sampling kernels
                         * advance it by the blocks their draws consumed       */
  double* stats;        /* [n_stat_slots][4]: result, sigma2, points, unused   */
  int64_t n_stat_slots; /* rows of stats                                       */
  int32_t* flags;       /* [8]: [0] map updates skipped (all-zero weights),
                         * [1] infinite edges repaired, [2] unrepairable edges,
                         * [3] a finish found its slot >= n_stat_slots      */
  double* scalars;      /* [4]: [0] sum of the unnormalised dh              */
  const void* domain;   /* [d][2] dtype                                        */
  int64_t* control;     /* [16] per-iteration inputs read by the kernels, so
                         * a sequence of launches can be captured once and
                         * replayed: [0] nevals_exp (VEGAS._starting_N),
                         * [1] statistics slot of the next finish (advanced by
                         * tq_vegas_finish_iteration), [2] 1 if dh awaits
                         * normalisation (set by finish, cleared by get_nh),
                         * [3] Philox seed, [4] Philox stream id; the loop
                         * state of tq_vegas_begin_run/tq_vegas_abort_test:
                         * [5] N, [6] N_increment, [7] max_iterations,
                         * [8] eps_rel, [9] eps_abs (IEEE double bits),
                         * [10] warm-up evaluations, [11] iterations done,
                         * [12] stop reason (0 go on, 1 accuracy reached,
                         * 2 evaluation budget, 3 iteration limit, 4 out of
                         * statistics slots, 5 / 6 int() of an infinite / NaN
                         * value, where the reference raises), [13]
                         * evaluations so far,
                         * [14] 1 while cube_start is split (see
                         * tq_vegas_get_nh_split)                          */
} tq_vegas_state;

enum {
  TQ_VC_NEVALS = 1,
  TQ_VC_SLOT = 2,
  TQ_VC_NORMALIZE = 4,
  TQ_VC_SEED = 8,
  TQ_VC_STREAM = 16
};

/* Scratch bytes the VEGAS entry points need for this state. */
size_t tq_vegas_workspace_size(const tq_vegas_state* st);

/* VEGASMap.__init__/_reset_weight (vegas_map.py:15-42,174-183) and the
 * initial VEGASStratification.dh (vegas_stratification.py:13-44). */
int tq_vegas_init(const tq_vegas_state* st, void* stream);

/* Writes the control fields selected by `mask` (TQ_VC_* bits) on the stream
 * (a one-thread kernel, so it orders with the other launches). */
int tq_vegas_set_control(const tq_vegas_state* st, int mask, int64_t nevals_exp, int64_t slot,
                         int64_t normalize, uint64_t seed, uint64_t stream_id, void* stream);

/* ---- the iteration loop on the device (tq_vegas_loop.cu) -------------------
 * VEGAS.integrate's loop (vegas.py:141-160): blocks of five iterations, then
 * _check_abort_conditions (:161-209), until it says stop.  With these two
 * calls and the capture helpers below a whole integration is one CUDA graph:
 * warm-up, then a WHILE node whose body is a block plus tq_vegas_abort_test. */
typedef struct {
  int64_t nevals_exp;     /* VEGAS._starting_N of the first block            */
  int64_t N;              /* evaluation budget                                */
  int64_t N_increment;    /* VEGAS._N_increment                               */
  int64_t max_iterations;
  int64_t warm_evals;     /* evaluations spent by the warm-up                 */
  double eps_rel, eps_abs;
  uint64_t seed, stream_id; /* Philox key and stream of the run              */
  uint64_t rng_offset;    /* Philox block offset the run starts at           */
  int32_t n_params;       /* entries of params copied to params_dev           */
  int32_t n_domain;       /* 0, or 2*dim: domain values for st->domain        */
  double params[2 + 2 * TQ_MAX_DIM]; /* built-in integrand parameters      */
  double domain[2 * TQ_MAX_DIM];     /* [dim][2] bounds, rounded to the
                                      * state's dtype when written         */
} tq_vegas_run;

/* The per-call inputs of a run in one one-thread launch: control [0], [3..10]
 * from `run`, [11..12] = 0, [13] = warm_evals; *st->rng_offset;
 * run->params[0..n_params) into params_dev (the parameter vector the fused
 * kernels read); and, if n_domain = 2*dim, the domain into st->domain (so a
 * domain given as host values needs no copy of its own). */
int tq_vegas_begin_run(const tq_vegas_state* st, const tq_vegas_run* run, double* params_dev,
                       void* stream);

/* _check_abort_conditions with _get_result, _get_error and _get_chisq
 * (vegas.py:161-209, 318-362) after a block of five iterations, on the
 * device in fp64: reads the block's five statistics rows (result, variance)
 * ending at control[1], sets control[13] = warm-up + points of all
 * iterations, control[11] += 5, control[12] = stop reason, and adapts
 * control[0] (nevals_exp) as the reference adapts _starting_N.  Every sum is
 * taken left to right from zero and x / 0 follows IEEE, as in the
 * reference's tensor arithmetic.  cond_handle != 0: the
 * cudaGraphConditionalHandle of the WHILE node this runs in, set to 0 to
 * stop. */
int tq_vegas_abort_test(const tq_vegas_state* st, uint64_t cond_handle, void* stream);

/* ---- many VEGAS states per launch (tq_vegas_batch.cu) ---------------------
 * A batch of resident VEGAS states advanced together: each phase of the
 * fused integration (the launches a single state's graph makes, see
 * tq_vegas_begin_run .. tq_vegas_abort_test) is one launch for every state
 * of the batch, whose CTAs are split among the states in proportion to
 * their work.  No counterpart in the reference, whose VEGAS.integrate
 * (vegas.py:100-160) runs one integral per call; each state follows the
 * reference's algorithm exactly as a single fused run does.  States of a
 * batch share the dtype; maps have at most 1024 intervals per dimension. */
enum {
  TQ_VB_BEGIN = 0,      /* the run inputs (runs[i]) and the state reset      */
  TQ_VB_WARM = 1,       /* one warm-up sampling pass                         */
  TQ_VB_MAP = 2,        /* the warm-up map update (one CTA per dimension)    */
  TQ_VB_NH = 3,         /* get_NH, cube prefix left split                    */
  TQ_VB_SAMPLE = 4,     /* one stratified sampling iteration                 */
  TQ_VB_FINISH = 5,     /* end of the iteration, beside the map update       */
  TQ_VB_ABORT = 6,      /* the abort test after a block of five iterations;
                         * the last CTA sets the graph condition: 1 while some
                         * state goes on                                     */
  TQ_VB_PHASES = 7
};

/* One state of a batch. */
typedef struct tq_vegas_item {
  tq_vegas_state st;        /* the state (its arrays in device memory)        */
  double* params;           /* [2 + 2 dim] device: the integrand parameters
                             * the run writes and the samplers read          */
  void* workspace;          /* tq_vegas_workspace_size(&st) device bytes      */
  size_t workspace_bytes;
  int64_t warm_samples;     /* points per warm-up pass (0: no warm-up)        */
  int64_t expected_points;  /* points of an iteration, sizes its CTA share    */
  int32_t family;           /* TQ_FN_* (built-in integrand)                   */
  int32_t use_grid_improve; /* map histogram and map update per iteration     */
  int32_t use_warmup;       /* five warm-up passes with map updates          */
  int32_t pad;
} tq_vegas_item;

/* What the launches of a batch need on the host (filled by
 * tq_vegas_batch_build). */
typedef struct tq_vegas_batch_info {
  int64_t n_items;
  int32_t dtype;
  int32_t pad;
  int64_t ctas[TQ_VB_PHASES]; /* CTAs of each phase's launch                 */
  int64_t smem[TQ_VB_PHASES]; /* dynamic shared memory of each launch        */
} tq_vegas_batch_info;

/* Device bytes of the table of the batch items[n_items] (host); 0 if an
 * item is invalid. */
size_t tq_vegas_batch_table_size(const tq_vegas_item* items, int64_t n_items);

/* Checks items[n_items] (host), builds the batch's table in `table` (device,
 * tq_vegas_batch_table_size bytes; copied on `stream`, which is then
 * synchronised) and fills *info. */
int tq_vegas_batch_build(const tq_vegas_item* items, int64_t n_items, void* table, size_t table_bytes,
                         tq_vegas_batch_info* info, void* stream);

/* Runs `phase` for every state of the batch in one launch.  runs[n_items]
 * (device; TQ_VB_BEGIN only): each state's run inputs, as
 * tq_vegas_begin_run takes them (at most 2 + 2 dim parameters are copied,
 * and the domain only when n_domain is 2 dim).  States stopped by their
 * abort test (control[12] != 0) skip TQ_VB_NH .. TQ_VB_ABORT.  cond_handle (ABORT):
 * the cudaGraphConditionalHandle of the WHILE node the launch runs in, or 0. */
int tq_vegas_batch_phase(const tq_vegas_batch_info* info, const void* table, int phase,
                         const tq_vegas_run* runs, double alpha, double beta, uint64_t cond_handle,
                         void* stream);


/* Capture helpers for a device-side loop (CUDA graph conditional nodes).
 * During a stream capture on `stream`, tq_capture_while_begin appends a
 * WHILE node (condition 1 at every graph launch) after the captured work,
 * makes it the stream's capture dependency and starts capturing the node's
 * body on body_stream (another, idle stream of the device); *cond_handle
 * receives the node's handle.  tq_capture_while_end ends the body capture;
 * the capture on `stream` goes on after the node. */
int tq_capture_while_begin(void* stream, void* body_stream, uint64_t* cond_handle);
int tq_capture_while_end(void* body_stream);

/* One warm-up iteration, fused (vegas.py:228-256 without the map update):
 * y = u * 0.999999 with u from the Philox stream (control seed and stream
 * id, block offset *st->rng_offset), x = map(y), f = integrand(domain(x)) *
 * volume, accumulate (f*jac)^2 into the map.  Advances *st->rng_offset. */
int tq_vegas_warmup_fused(const tq_vegas_state* st, int family, const double* params,
                          int64_t n_samples, void* workspace, size_t workspace_bytes,
                          void* stream);

/* VEGASMap.update_map (vegas_map.py:185-261) incl. _smooth_map (:113-172);
 * resets weights and counts.  Sets flags[0] if a dimension's weights are all
 * zero (map left unchanged), flags[1]/[2] for repaired/unrepairable
 * infinite edges. */
int tq_vegas_update_map(const tq_vegas_state* st, double alpha, void* workspace,
                        size_t workspace_bytes, void* stream);

/* VEGASMap._smooth_map (vegas_map.py:113-172) alone: writes the smoothed,
 * range-compressed weights [d][B] (dtype) of the current weights/counts to
 * `smoothed`; map, weights and counts are left unchanged. */
int tq_vegas_smooth_weights(const tq_vegas_state* st, double alpha, void* smoothed,
                            void* workspace, size_t workspace_bytes, void* stream);

/* VEGASStratification.get_NH (vegas_stratification.py:92-103):
 * neval = max(2, floor(dh * control[0])), cube_start = exclusive prefix,
 * cube_start[n_cubes] = total; zeroes jf/jf2.  If control[2] != 0 the dh
 * left unnormalised by tq_vegas_finish_iteration is first divided by its sum
 * (vegas_stratification.py:88-90) and control[2] is cleared. */
int tq_vegas_get_nh(const tq_vegas_state* st, void* workspace, size_t workspace_bytes,
                    void* stream);
/* get_NH without the fix-up launch: cube_start is left split (each
 * 256-cube block's prefix local to the block, the block offsets in the
 * workspace) and control[14] = 1.  tq_vegas_iterate_fused adds the offsets
 * where it reads cube_start, and tq_vegas_finish_iteration (or
 * tq_vegas_finish_update_map) writes them back and clears control[14].  For
 * sequences that run exactly get_NH, the fused sampling and finish. */
int tq_vegas_get_nh_split(const tq_vegas_state* st, void* workspace, size_t workspace_bytes,
                          void* stream);

/* One stratified iteration, fused (vegas.py:274-291): for every point of
 * every cube (cube_start order), y = (cube position + u) / n_strat
 * (get_Y, vegas_stratification.py:140-165), x and jac from the map
 * (get_X/get_Jac, vegas_map.py:44-74), f = integrand(domain(x)) * volume;
 * accumulates the map weights/counts (if use_grid_improve) and the per-cube
 * sums jf/jf2 (accumulate_weight, vegas_stratification.py:46-70).
 * max_points sizes the launch: about two 32-point tiles per warp for that
 * many points, at most one full wave of CTAs (0: one full wave); any count
 * of points is covered whatever the size.  Advances *st->rng_offset. */
int tq_vegas_iterate_fused(const tq_vegas_state* st, int family, const double* params,
                           int use_grid_improve, int64_t max_points, void* workspace,
                           size_t workspace_bytes, void* stream);

/* Per-cube estimates -> stats[control[1]] = {sum ih, sum sig2/n, points}
 * (vegas.py:293-303, fp64 compensated sums) and the unnormalised dampened
 * counts dh (update_DH, vegas_stratification.py:72-90; the division by the
 * sum happens in the next tq_vegas_get_nh).  Advances control[1] and sets
 * control[2].  The caller keeps control[1] below the rows of stats. */
int tq_vegas_finish_iteration(const tq_vegas_state* st, double beta, void* workspace,
                              size_t workspace_bytes, void* stream);

/* tq_vegas_finish_iteration followed by tq_vegas_update_map (the end of one
 * stratified iteration with the map improved, vegas.py:303 then
 * vegas.py:313 -> vegas_map.py:185-261).  For maps of at most 1024
 * intervals per dimension both run in one launch side by side (they touch
 * disjoint parts of the state); larger maps take the two calls. */
int tq_vegas_finish_update_map(const tq_vegas_state* st, double beta, double alpha,
                               void* workspace, size_t workspace_bytes, void* stream);

/* Materialised path (arbitrary torch integrands, injected uniforms). */

/* y[M][d] = stratified points from uniforms u[M][d] (get_Y); M must equal
 * cube_start[n_cubes]. */
int tq_vegas_strat_points(const tq_vegas_state* st, const void* u, int64_t n_points, void* y,
                          void* stream);
/* x[M][d] = map(y), jac[M] = Jacobian (get_X, get_Jac), both dtype. */
int tq_vegas_map_points(const tq_vegas_state* st, const void* y, int64_t n_points, void* x,
                        void* jac, void* stream);
/* accumulate_map: weights[k][ID_k(y)] += vals, counts += 1
 * (VEGASMap.accumulate_weight, vegas_map.py:99-111, which receives (f*jac)^2);
 * stratified: jf[c] += vals, jf2[c] += vals^2 over the cubes in cube_start
 * order (VEGASStratification.accumulate_weight, :46-70, which receives
 * f*jac).  vals is dtype [M]. */
int tq_vegas_accumulate(const tq_vegas_state* st, const void* y, const void* vals,
                        int64_t n_points, int accumulate_map, int stratified,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ---- measurement ---------------------------------------------------------- */

/* FP32 FMA throughput probe (no reference counterpart; used by the benchmark
 * to measure the FP32 roofline): launches sm_count*blocks_per_sm CTAs doing
 * iters*128 dependent-free FMAs per thread; *flops receives the flop count. */
int tq_fp32_fma_probe(int64_t iters, int blocks_per_sm, float* out, double* flops,
                      void* stream);

/* The same with fp64 fused multiply-adds: the FP64-pipe peak the fp64 grid
 * kernels are measured against (out: one double). */
int tq_fp64_fma_probe(int64_t iters, int blocks_per_sm, double* out, double* flops, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TORCHQUAD_GB300_H */
