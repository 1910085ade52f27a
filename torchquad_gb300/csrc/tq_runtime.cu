// Status plumbing and device queries shared by every entry point.
#include <atomic>

#include "tq_common.cuh"

namespace tq {

static thread_local int g_last_cuda_error = 0;

int set_cuda_error(cudaError_t e) {
  g_last_cuda_error = (int)e;
  return TQ_ERR_CUDA;
}

int launch_status() {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TQ_OK : set_cuda_error(e);
}

static std::atomic<int> g_sm_count[64];

int sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int v = g_sm_count[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
    v = 152;
  g_sm_count[dev].store(v, std::memory_order_relaxed);
  return v;
}

}  // namespace tq

extern "C" const char* tq_status_string(int status) {
  switch (status) {
    case TQ_OK:
      return "ok";
    case TQ_ERR_ARG:
      return "invalid argument (null pointer or inconsistent sizes)";
    case TQ_ERR_DIM:
      return "dimension out of range for this kernel";
    case TQ_ERR_RULE:
      return "unknown quadrature rule or point count invalid for the rule";
    case TQ_ERR_FAMILY:
      return "unknown built-in integrand family";
    case TQ_ERR_TOO_LARGE:
      return "problem size overflows the index arithmetic";
    case TQ_ERR_WORKSPACE:
      return "workspace smaller than the size query returned";
    case TQ_ERR_CUDA:
      return "CUDA runtime error (see tq_last_cuda_error)";
    case TQ_ERR_DTYPE:
      return "unknown dtype code";
    case TQ_ERR_TIMEOUT:
      return "a bounded device-side wait gave up";
    case TQ_ERR_SCRATCH:
      return "problem needs more scratch than the static buffer of the allocation-free entry point holds";
    default:
      return "unknown status";
  }
}

extern "C" int tq_last_cuda_error(void) { return tq::g_last_cuda_error; }

extern "C" int tq_device_sm_count(void) { return tq::sm_count(); }
