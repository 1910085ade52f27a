// The VEGAS iteration loop on the device: the per-call inputs of a run and
// the abort test after every fifth iteration, so that a whole integration
// (warm-up, then blocks of five iterations while the test says go on) is
// one CUDA graph with a WHILE conditional node and no host round trip.
//
// Reference (torchquad v0.5.0): vegas.py:100-209 (VEGAS.integrate and
// _check_abort_conditions), :318-362 (_get_result, _get_error, _get_chisq).

#include "tq_vegas_control.cuh"

namespace tq {

__global__ void vegas_begin_run_kernel(RunArgs a) { begin_run_body(a); }

__global__ void __launch_bounds__(32) vegas_abort_kernel(AbortArgs a) { abort_body(a); }

}  // namespace tq

using namespace tq;

extern "C" int tq_vegas_begin_run(const tq_vegas_state* st, const tq_vegas_run* run,
                                  double* params_dev, void* stream) {
  if (!st || !run || !st->control || !st->rng_offset) return TQ_ERR_ARG;
  if (run->n_params < 0 || run->n_params > 2 + 2 * TQ_MAX_DIM || (run->n_params > 0 && !params_dev))
    return TQ_ERR_ARG;
  if (run->max_iterations < 0 || run->N < 0 || run->N_increment < 0 || run->nevals_exp < 0)
    return TQ_ERR_ARG;
  if (run->n_domain != 0 && (run->n_domain != 2 * st->dim || !st->domain || !valid_dtype(st->dtype)))
    return TQ_ERR_ARG;
  RunArgs a;
  memcpy(&a.run, run, sizeof(tq_vegas_run));
  a.control = st->control;
  a.rng_offset = st->rng_offset;
  a.params_dev = params_dev;
  a.domain = const_cast<void*>(st->domain);
  a.dtype = st->dtype;
  vegas_begin_run_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(a);
  return launch_status();
}

extern "C" int tq_vegas_abort_test(const tq_vegas_state* st, uint64_t cond_handle, void* stream) {
  if (!st || !st->control || !st->stats || st->n_stat_slots < 1) return TQ_ERR_ARG;
  AbortArgs a;
  a.control = st->control;
  a.dtype = st->dtype;
  a.stats = st->stats;
  a.n_stat_slots = st->n_stat_slots;
  a.handle = (cudaGraphConditionalHandle)cond_handle;
  a.use_handle = cond_handle != 0;
  vegas_abort_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(a);
  return launch_status();
}

extern "C" int tq_capture_while_begin(void* stream, void* body_stream, uint64_t* cond_handle) {
  if (!cond_handle || stream == body_stream) return TQ_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus status;
  cudaGraph_t graph = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t n_deps = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(s, &status, nullptr, &graph, &deps, &edges, &n_deps);
  if (e != cudaSuccess) return set_cuda_error(e);
  if (status == cudaStreamCaptureStatusInvalidated) return set_cuda_error(cudaErrorStreamCaptureInvalidated);
  if (status != cudaStreamCaptureStatusActive || !graph) return TQ_ERR_ARG;
  cudaGraphConditionalHandle h;
  e = cudaGraphConditionalHandleCreate(&h, graph, 1u, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return set_cuda_error(e);
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, graph, deps, edges, n_deps, &p);
  if (e != cudaSuccess) return set_cuda_error(e);
  e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  if (e != cudaSuccess) return set_cuda_error(e);
  e = cudaStreamBeginCaptureToGraph((cudaStream_t)body_stream, p.conditional.phGraph_out[0], nullptr,
                                    nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return set_cuda_error(e);
  *cond_handle = (uint64_t)h;
  return TQ_OK;
}

extern "C" int tq_capture_while_end(void* body_stream) {
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture((cudaStream_t)body_stream, &g);
  return e == cudaSuccess ? TQ_OK : set_cuda_error(e);
}
