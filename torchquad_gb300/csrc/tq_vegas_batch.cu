// Many resident VEGAS states advanced together: each phase of a fused VEGAS
// integration (state reset and run inputs, warm-up sampling, warm-up map
// update, get_NH, stratified sampling, end of iteration beside the map
// update, abort test) is one launch for the whole batch.  A phase's CTAs
// are split among the states in proportion to their work; a table built
// once on the host maps every CTA to (state, CTA index within the state),
// and the CTA runs the same device body (tq_vegas_phases.cuh,
// tq_vegas_sample.cuh, tq_vegas_control.cuh) that the single-state kernels
// run with that state's arguments.  So each state follows the reference's
// algorithm exactly as its own fused run does, and a captured graph of the
// phases (a WHILE node around blocks of five iterations) integrates the
// whole batch with one launch per phase instead of one per state.
//
// Reference (torchquad v0.5.0): vegas.py:100-209 (VEGAS.integrate, one
// integral per call), vegas_map.py, vegas_stratification.py.

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "tq_vegas_control.cuh"
#include "tq_vegas_phases.cuh"

namespace tq {

constexpr int kBatchAbortThreads = 32;
constexpr int64_t kBatchInitCtas = 64;
// Dynamic shared memory of a batched sampling launch (the largest state's):
// four fp32 sampler CTAs (64 registers a thread), or three fp64 ones (85),
// fit an SM's 228 KB.
constexpr size_t kBatchSampleSmem = 56 * 1024;
constexpr size_t kBatchSampleSmemF64 = 72 * 1024;

// One state of the batch: the arguments of every phase body, built on the
// host by the same helpers the single-state launchers use.
struct BatchEntry {
  tq_vegas_state st;
  SampleArgs warm;  // warm-up sampling (n_samples = warm-up points)
  SampleArgs iter;  // stratified sampling
  NhArgs nh;
  FinishArgs fin;
  double* params;
  unsigned* t_map;
  int32_t ctas[TQ_VB_PHASES];
  int32_t map_rows;  // CTAs of the FINISH phase that update the map (0 or dim)
  int32_t pad;
};

// Table header; the ticket and counter of the ABORT phase's condition.
struct BatchHeader {
  unsigned ticket;
  unsigned active;    // states still going on, counted during ABORT
  unsigned last_active;  // the count of the last ABORT (read by the host)
  unsigned pad;
  int64_t n_items;
  int64_t entries;                 // byte offset of BatchEntry[n_items]
  int64_t map[TQ_VB_PHASES];       // byte offset of each phase's uint2 [ctas]
};

struct BatchLaunch {
  BatchHeader* hdr;
  const BatchEntry* e;
  const uint2* map;  // (state, CTA within the state) per CTA of this phase
  const tq_vegas_run* runs;
  double alpha, beta;
  cudaGraphConditionalHandle handle;
  int use_handle;
};

__device__ __forceinline__ bool batch_stopped(const BatchEntry& e) {
  return __ldcg(e.st.control + kCtlStop) != 0;
}

template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_batch_begin_kernel(BatchLaunch L) {
  const uint2 m = L.map[blockIdx.x];
  const BatchEntry& e = L.e[m.x];
  if (m.y == 0 && threadIdx.x == 0)
    begin_run_from(L.runs[m.x], e.st.control, e.st.rng_offset, e.params, const_cast<void*>(e.st.domain),
                   e.st.dtype, 2 + 2 * e.st.dim, 2 * e.st.dim);
  init_body<T>(e.st, m.y, (unsigned)e.ctas[TQ_VB_BEGIN]);
}

template <typename T, bool WARM>
__device__ __forceinline__ void batch_sample(const SampleArgs& a, int family, unsigned bid, unsigned nblk) {
  switch (family) {
    case TQ_FN_EXP_SUM:
      sample_body<T, TQ_FN_EXP_SUM, WARM, 0>(a, bid, nblk);
      break;
    case TQ_FN_GAUSSIAN:
      sample_body<T, TQ_FN_GAUSSIAN, WARM, 0>(a, bid, nblk);
      break;
    case TQ_FN_OSCILLATORY:
      sample_body<T, TQ_FN_OSCILLATORY, WARM, 0>(a, bid, nblk);
      break;
    default:
      sample_body<T, TQ_FN_SUM_SIN, WARM, 0>(a, bid, nblk);
      break;
  }
}

template <typename T, bool WARM>
__global__ void __launch_bounds__(kTile, std::is_same<T, double>::value ? 3 : TQ_SAMPLE_MIN_BLOCKS)
    vegas_batch_sample_kernel(BatchLaunch L) {
  const uint2 m = L.map[blockIdx.x];
  const BatchEntry& e = L.e[m.x];
  if (!WARM && batch_stopped(e)) return;
  const SampleArgs a = WARM ? e.warm : e.iter;  // a private copy the compiler may keep in registers
  batch_sample<T, WARM>(a, a.family, m.y, (unsigned)e.ctas[WARM ? TQ_VB_WARM : TQ_VB_SAMPLE]);
}

template <typename T>
__device__ __forceinline__ void batch_map_row(const BatchEntry& e, double alpha, int k, unsigned nrows) {
  if constexpr (std::is_same<T, float>::value)
    map_rows_f32_body(e.st, alpha, nullptr, e.t_map, k, nrows);
  else
    map_rows_body<T>(e.st, alpha, nullptr, e.t_map, k, nrows);
}

template <typename T>
__global__ void __launch_bounds__(kRowThreads) vegas_batch_map_kernel(BatchLaunch L) {
  const uint2 m = L.map[blockIdx.x];
  const BatchEntry& e = L.e[m.x];
  batch_map_row<T>(e, L.alpha, (int)m.y, (unsigned)e.ctas[TQ_VB_MAP]);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_batch_nh_kernel(BatchLaunch L) {
  const uint2 m = L.map[blockIdx.x];
  const BatchEntry& e = L.e[m.x];
  if (batch_stopped(e)) return;
  nh_body<T>(e.nh, m.y, (unsigned)e.ctas[TQ_VB_NH]);
}

// CTAs [0, map_rows) of a state update its map rows, the others end its
// iteration (the two touch disjoint parts of the state).
template <typename T>
__global__ void __launch_bounds__(kBlock) vegas_batch_finish_kernel(BatchLaunch L) {
  const uint2 m = L.map[blockIdx.x];
  const BatchEntry& e = L.e[m.x];
  if (batch_stopped(e)) return;
  const unsigned rows = (unsigned)e.map_rows;
  if (m.y < rows) {
    batch_map_row<T>(e, L.alpha, (int)m.y, rows);
  } else {
    const unsigned nblk = (unsigned)e.ctas[TQ_VB_FINISH] - rows;
    FinishArgs a = e.fin;
    a.beta = L.beta;
    if constexpr (std::is_same<T, float>::value)
      finish_f32_body(a, m.y - rows, nblk);
    else
      finish_body<T>(a, m.y - rows, nblk);
  }
}

// One warp per state.  The last CTA to finish sets the WHILE condition: 1
// while some state goes on.
__global__ void __launch_bounds__(kBatchAbortThreads) vegas_batch_abort_kernel(BatchLaunch L) {
  const BatchEntry& e = L.e[blockIdx.x];
  const bool was_running = !batch_stopped(e);
  if (was_running) {
    AbortArgs a;
    a.control = e.st.control;
    a.dtype = e.st.dtype;
    a.stats = e.st.stats;
    a.n_stat_slots = e.st.n_stat_slots;
    a.handle = 0;
    a.use_handle = 0;
    abort_body(a);  // lane 0 writes the stop reason
  }
  if (threadIdx.x == 0 && was_running && e.st.control[kCtlStop] == 0) atomicAdd(&L.hdr->active, 1u);
  if (last_block_of(&L.hdr->ticket, gridDim.x) && threadIdx.x == 0) {
    const unsigned n = atomicExch(&L.hdr->active, 0u);
    L.hdr->last_active = n;
    L.hdr->ticket = 0u;
    if (L.use_handle) cudaGraphSetConditional(L.handle, n > 0 ? 1u : 0u);
  }
}

}  // namespace tq

using namespace tq;

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int64_t clamp_ctas(int64_t x, int64_t hi) { return x < 1 ? 1 : (x > hi ? hi : x); }

struct BatchLayout {
  size_t entries, map[TQ_VB_PHASES], total;
  int64_t ctas[TQ_VB_PHASES];
};

// The CTA share of each phase for one item, and the item checks.
int item_ctas(const tq_vegas_item& it, int32_t ctas[TQ_VB_PHASES], int32_t* map_rows) {
  const tq_vegas_state* st = &it.st;
  const int rc = vegas_check_state(st);
  if (rc != TQ_OK) return rc;
  if (st->n_bins > kSmallMap) return TQ_ERR_TOO_LARGE;
  if (!it.params || !it.workspace || it.warm_samples < 0 || it.expected_points < 0) return TQ_ERR_ARG;
  if (it.workspace_bytes < vegas_workspace_view(st, nullptr).total) return TQ_ERR_WORKSPACE;
  if (it.family < TQ_FN_EXP_SUM || it.family > TQ_FN_SUM_SIN) return TQ_ERR_FAMILY;
  const int64_t work = st->n_cubes > st->dim * (st->n_bins + 1) ? st->n_cubes : st->dim * (st->n_bins + 1);
  ctas[TQ_VB_BEGIN] = (int32_t)clamp_ctas((work + kBlock - 1) / kBlock, kBatchInitCtas);
  ctas[TQ_VB_WARM] = (it.use_warmup && it.warm_samples > 0) ? (int32_t)vegas_sample_ctas(st, it.warm_samples) : 0;
  ctas[TQ_VB_MAP] = it.use_warmup ? st->dim : 0;
  const int64_t nh = vegas_nh_blocks(st);
  if (nh > (int64_t(1) << 24)) return TQ_ERR_TOO_LARGE;
  ctas[TQ_VB_NH] = (int32_t)nh;
  ctas[TQ_VB_SAMPLE] = (int32_t)vegas_sample_ctas(st, it.expected_points);
  *map_rows = it.use_grid_improve ? st->dim : 0;
  ctas[TQ_VB_FINISH] = (int32_t)(*map_rows + vegas_finish_blocks(st));
  ctas[TQ_VB_ABORT] = 1;
  return TQ_OK;
}

int batch_layout(const tq_vegas_item* items, int64_t n, BatchLayout* L) {
  if (!items || n < 1 || n > (int64_t(1) << 24)) return TQ_ERR_ARG;
  for (int p = 0; p < TQ_VB_PHASES; ++p) L->ctas[p] = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (items[i].st.dtype != items[0].st.dtype) return TQ_ERR_DTYPE;
    int32_t c[TQ_VB_PHASES], rows;
    const int rc = item_ctas(items[i], c, &rows);
    if (rc != TQ_OK) return rc;
    for (int p = 0; p < TQ_VB_PHASES; ++p) L->ctas[p] += c[p];
  }
  for (int p = 0; p < TQ_VB_PHASES; ++p)
    if (L->ctas[p] > 0x7fffffff) return TQ_ERR_TOO_LARGE;
  size_t off = align256(sizeof(BatchHeader));
  L->entries = off;
  off += align256(sizeof(BatchEntry) * (size_t)n);
  for (int p = 0; p < TQ_VB_PHASES; ++p) {
    L->map[p] = off;
    off += align256(sizeof(uint2) * (size_t)L->ctas[p]);
  }
  L->total = off;
  return TQ_OK;
}

}  // namespace

extern "C" size_t tq_vegas_batch_table_size(const tq_vegas_item* items, int64_t n_items) {
  BatchLayout L;
  return batch_layout(items, n_items, &L) == TQ_OK ? L.total : 0;
}

extern "C" int tq_vegas_batch_build(const tq_vegas_item* items, int64_t n_items, void* table,
                                    size_t table_bytes, tq_vegas_batch_info* info, void* stream) {
  BatchLayout L;
  int rc = batch_layout(items, n_items, &L);
  if (rc != TQ_OK) return rc;
  if (!table || !info) return TQ_ERR_ARG;
  if (table_bytes < L.total) return TQ_ERR_WORKSPACE;
  std::vector<unsigned char> host(L.total, 0);
  BatchHeader* h = (BatchHeader*)host.data();
  h->n_items = n_items;
  h->entries = (int64_t)L.entries;
  for (int p = 0; p < TQ_VB_PHASES; ++p) h->map[p] = (int64_t)L.map[p];
  BatchEntry* ents = (BatchEntry*)(host.data() + L.entries);
  int64_t cursor[TQ_VB_PHASES] = {0};
  size_t smem_sample = 0, smem_warm = 0;
  int64_t max_bins = 2;
  const size_t edges_limit = items[0].st.dtype == TQ_F64 ? kBatchSampleSmemF64 : kBatchSampleSmem;
  for (int64_t i = 0; i < n_items; ++i) {
    const tq_vegas_item& it = items[i];
    const tq_vegas_state* st = &it.st;
    BatchEntry& e = ents[i];
    memcpy(&e.st, st, sizeof(tq_vegas_state));
    item_ctas(it, e.ctas, &e.map_rows);
    const VegasWsView ws = vegas_workspace_view(st, it.workspace);
    size_t sm = 0;
    e.warm = vegas_sample_args(st, it.family, it.params, it.warm_samples > 0 ? it.warm_samples : 1, 1,
                               ws.t_sample, nullptr, &sm, edges_limit);
    if (e.ctas[TQ_VB_WARM] > 0 && sm > smem_warm) smem_warm = sm;
    e.iter = vegas_sample_args(st, it.family, it.params, 0, it.use_grid_improve ? 1 : 0, ws.t_sample,
                               ws.block_tot, &sm, edges_limit);
    if (sm > smem_sample) smem_sample = sm;
    e.nh.st = *st;
    e.nh.block_tot = ws.block_tot;
    e.nh.ticket = ws.t_nh;
    e.nh.split = 1;
    e.fin.st = *st;
    e.fin.beta = 0.0;  // the launch's beta replaces it
    e.fin.V = pow(1.0 / (double)st->n_strat, (double)st->dim);
    e.fin.partials = ws.partials;
    e.fin.ticket = ws.t_finish;
    e.fin.block_pre = ws.block_tot;
    e.params = it.params;
    e.t_map = ws.t_map;
    if (st->n_bins > max_bins) max_bins = st->n_bins;
  }
  // CTAs in order of integrand family and dimension: the CTAs resident on
  // an SM at once then mostly run the same code (one instantiation of the
  // sampler per family), which keeps the instruction cache warm
  std::vector<int64_t> order((size_t)n_items);
  for (int64_t i = 0; i < n_items; ++i) order[(size_t)i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
    if (items[x].family != items[y].family) return items[x].family < items[y].family;
    return items[x].st.dim < items[y].st.dim;
  });
  for (const int64_t i : order) {
    const BatchEntry& e = ents[i];
    for (int p = 0; p < TQ_VB_PHASES; ++p) {
      uint2* m = (uint2*)(host.data() + L.map[p]);
      for (int32_t c = 0; c < e.ctas[p]; ++c) m[cursor[p] + c] = make_uint2((unsigned)i, (unsigned)c);
      cursor[p] += e.ctas[p];
    }
  }
  const size_t ts = dtype_size(items[0].st.dtype);
  info->n_items = n_items;
  info->dtype = items[0].st.dtype;
  info->pad = 0;
  for (int p = 0; p < TQ_VB_PHASES; ++p) {
    info->ctas[p] = L.ctas[p];
    info->smem[p] = 0;
  }
  info->smem[TQ_VB_WARM] = (int64_t)smem_warm;
  info->smem[TQ_VB_SAMPLE] = (int64_t)smem_sample;
  info->smem[TQ_VB_MAP] = (int64_t)map_row_smem(max_bins, ts);
  info->smem[TQ_VB_FINISH] = (int64_t)map_row_smem(max_bins, ts);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(table, host.data(), L.total, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? TQ_OK : set_cuda_error(e);
}

namespace {

template <typename K>
int launch_batch(K kfn, unsigned grid, unsigned threads, size_t smem, const BatchLaunch& L, cudaStream_t s) {
  const int rc = opt_in_smem(kfn, smem);
  if (rc != TQ_OK) return rc;
  kfn<<<grid, threads, smem, s>>>(L);
  return launch_status();
}

template <typename T>
int batch_phase(const tq_vegas_batch_info* info, const void* table, int phase, const tq_vegas_run* runs,
                double alpha, double beta, uint64_t cond_handle, cudaStream_t s) {
  // The header's offsets are the host's own layout of the same items.
  unsigned char* base = (unsigned char*)const_cast<void*>(table);
  BatchLaunch L;
  L.hdr = (BatchHeader*)base;
  L.e = (const BatchEntry*)(base + align256(sizeof(BatchHeader)));
  size_t off = align256(sizeof(BatchHeader)) + align256(sizeof(BatchEntry) * (size_t)info->n_items);
  for (int p = 0; p < phase; ++p) off += align256(sizeof(uint2) * (size_t)info->ctas[p]);
  L.map = (const uint2*)(base + off);
  L.runs = runs;
  L.alpha = alpha;
  L.beta = beta;
  L.handle = (cudaGraphConditionalHandle)cond_handle;
  L.use_handle = cond_handle != 0;
  const unsigned grid = (unsigned)info->ctas[phase];
  const size_t smem = (size_t)info->smem[phase];
  if (grid == 0) return TQ_OK;
  switch (phase) {
    case TQ_VB_BEGIN:
      if (!runs) return TQ_ERR_ARG;
      return launch_batch(vegas_batch_begin_kernel<T>, grid, kBlock, 0, L, s);
    case TQ_VB_WARM:
      return launch_batch(vegas_batch_sample_kernel<T, true>, grid, kTile, smem, L, s);
    case TQ_VB_MAP:
      return launch_batch(vegas_batch_map_kernel<T>, grid, kRowThreads, smem, L, s);
    case TQ_VB_NH:
      return launch_batch(vegas_batch_nh_kernel<T>, grid, kBlock, 0, L, s);
    case TQ_VB_SAMPLE:
      return launch_batch(vegas_batch_sample_kernel<T, false>, grid, kTile, smem, L, s);
    case TQ_VB_FINISH:
      return launch_batch(vegas_batch_finish_kernel<T>, grid, kBlock, smem, L, s);
    case TQ_VB_ABORT:
      return launch_batch(vegas_batch_abort_kernel, grid, kBatchAbortThreads, 0, L, s);
    default:
      return TQ_ERR_ARG;
  }
}

}  // namespace

extern "C" int tq_vegas_batch_phase(const tq_vegas_batch_info* info, const void* table, int phase,
                                    const tq_vegas_run* runs, double alpha, double beta,
                                    uint64_t cond_handle, void* stream) {
  if (!info || !table || info->n_items < 1 || phase < 0 || phase >= TQ_VB_PHASES) return TQ_ERR_ARG;
  if (info->ctas[TQ_VB_ABORT] != info->n_items) return TQ_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (info->dtype == TQ_F64) return batch_phase<double>(info, table, phase, runs, alpha, beta, cond_handle, s);
  if (info->dtype == TQ_F32) return batch_phase<float>(info, table, phase, runs, alpha, beta, cond_handle, s);
  return TQ_ERR_DTYPE;
}
