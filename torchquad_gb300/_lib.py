"""ctypes binding of the C ABI declared in ``include/torchquad_gb300.h``.

The library is loaded on first use.  There is no fallback: if the library is
missing or no CUDA device is present, every integration call raises.
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER, c_double, c_int, c_int64, c_size_t, c_uint64, c_void_p, c_char_p

import torch

from .build import lib_path

# status codes (include/torchquad_gb300.h)
TQ_OK = 0
TQ_ERR_ARG = -1
TQ_ERR_DIM = -2
TQ_ERR_RULE = -3
TQ_ERR_FAMILY = -4
TQ_ERR_TOO_LARGE = -5
TQ_ERR_WORKSPACE = -6
TQ_ERR_CUDA = -7
TQ_ERR_DTYPE = -8
TQ_ERR_TIMEOUT = -9
TQ_ERR_SCRATCH = -10

TQ_F32, TQ_F64 = 0, 1

TQ_RULE_TRAPEZOID, TQ_RULE_SIMPSON, TQ_RULE_BOOLE, TQ_RULE_GAUSS, TQ_RULE_MC = 0, 1, 2, 3, 4

TQ_FN_EXP_SUM, TQ_FN_GAUSSIAN, TQ_FN_OSCILLATORY, TQ_FN_SUM_SIN = 1, 2, 3, 4
TQ_FN_PER_DESC = -1  # batched calls: each descriptor's own family

TQ_MAX_DIM = 16

class VegasState(ctypes.Structure):
    """Mirror of ``tq_vegas_state`` (include/torchquad_gb300.h)."""

    _fields_ = [
        ("dim", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("n_bins", c_int64),
        ("n_strat", c_int64),
        ("n_cubes", c_int64),
        ("x_edges", c_void_p),
        ("dx_edges", c_void_p),
        ("weights", c_void_p),
        ("counts", c_void_p),
        ("dh", c_void_p),
        ("jf", c_void_p),
        ("jf2", c_void_p),
        ("neval", c_void_p),
        ("cube_start", c_void_p),
        ("rng_offset", c_void_p),
        ("stats", c_void_p),
        ("n_stat_slots", c_int64),
        ("flags", c_void_p),
        ("scalars", c_void_p),
        ("domain", c_void_p),
        ("control", c_void_p),
    ]


TQ_VC_NEVALS, TQ_VC_SLOT, TQ_VC_NORMALIZE, TQ_VC_SEED, TQ_VC_STREAM = 1, 2, 4, 8, 16


class VegasRun(ctypes.Structure):
    """Mirror of ``tq_vegas_run`` (include/torchquad_gb300.h)."""

    _fields_ = [
        ("nevals_exp", c_int64),
        ("N", c_int64),
        ("N_increment", c_int64),
        ("max_iterations", c_int64),
        ("warm_evals", c_int64),
        ("eps_rel", c_double),
        ("eps_abs", c_double),
        ("seed", c_uint64),
        ("stream_id", c_uint64),
        ("rng_offset", c_uint64),
        ("n_params", ctypes.c_int32),
        ("n_domain", ctypes.c_int32),
        ("params", c_double * (2 + 2 * TQ_MAX_DIM)),
        ("domain", c_double * (2 * TQ_MAX_DIM)),
    ]


# control block fields of the device-side VEGAS loop (tq_vegas_state.control)
VC_NEVALS, VC_SLOT, VC_IT, VC_STOP, VC_EVALS = 0, 1, 11, 12, 13

# phases of a batch of VEGAS states (tq_vegas_batch_phase)
VB_BEGIN, VB_WARM, VB_MAP, VB_NH, VB_SAMPLE, VB_FINISH, VB_ABORT = range(7)
VB_PHASES = 7


class VegasItem(ctypes.Structure):
    """Mirror of ``tq_vegas_item`` (include/torchquad_gb300.h)."""

    _fields_ = [
        ("st", VegasState),
        ("params", c_void_p),
        ("workspace", c_void_p),
        ("workspace_bytes", c_size_t),
        ("warm_samples", c_int64),
        ("expected_points", c_int64),
        ("family", ctypes.c_int32),
        ("use_grid_improve", ctypes.c_int32),
        ("use_warmup", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class VegasBatchInfo(ctypes.Structure):
    """Mirror of ``tq_vegas_batch_info`` (include/torchquad_gb300.h)."""

    _fields_ = [
        ("n_items", c_int64),
        ("dtype", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("ctas", c_int64 * VB_PHASES),
        ("smem", c_int64 * VB_PHASES),
    ]


_VS = POINTER(VegasState)

# name -> (restype, argtypes); every symbol the header declares.
SIGNATURES = {
    "tq_status_string": (c_char_p, [c_int]),
    "tq_last_cuda_error": (c_int, []),
    "tq_device_sm_count": (c_int, []),
    "tq_grid_fused_workspace_size": (c_size_t, [c_int, c_int, c_int64]),
    "tq_grid_fused": (
        c_int,
        [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
         c_void_p, c_int, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "tq_grid_fused_noalloc": (
        c_int,
        [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
         c_void_p, c_int, c_void_p, c_void_p],
    ),
    "tq_grid_adjoint_workspace_size": (c_size_t, [c_int, c_int64]),
    "tq_grid_adjoint": (
        c_int,
        [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
         c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "tq_batch_grid_adjoint_workspace_size": (c_size_t, [c_int64, c_int]),
    "tq_batch_grid_adjoint": (
        c_int,
        [c_int, c_int64, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_void_p, c_void_p,
         c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "tq_batch_grid": (
        c_int,
        [c_int, c_int64, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_void_p, c_void_p,
         c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_size_t, c_void_p],
    ),
    "tq_batch_mc": (
        c_int,
        [c_int, c_int64, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_void_p, c_int, c_void_p,
         c_void_p, c_size_t, c_void_p],
    ),
    "tq_grid_points": (
        c_int,
        [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_void_p],
    ),
    "tq_grid_weights": (
        c_int,
        [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_void_p],
    ),
    "tq_weighted_sum_workspace_size": (c_size_t, [c_int64, c_int64]),
    "tq_weighted_sum": (
        c_int,
        [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_int,
         c_int64, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "tq_finalize_sum": (
        c_int,
        [c_int, c_int, c_int, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int, c_void_p],
    ),
    "tq_uniform": (c_int, [c_int, c_uint64, c_uint64, c_uint64, c_int64, c_void_p, c_void_p]),
    "tq_mc_fused_workspace_size": (c_size_t, [c_int, c_int64]),
    "tq_vegas_workspace_size": (c_size_t, [_VS]),
    "tq_vegas_init": (c_int, [_VS, c_void_p]),
    "tq_vegas_set_control": (c_int, [_VS, c_int, c_int64, c_int64, c_int64, c_uint64, c_uint64, c_void_p]),
    "tq_vegas_begin_run": (c_int, [_VS, POINTER(VegasRun), c_void_p, c_void_p]),
    "tq_vegas_abort_test": (c_int, [_VS, c_uint64, c_void_p]),
    "tq_vegas_batch_table_size": (c_size_t, [POINTER(VegasItem), c_int64]),
    "tq_vegas_batch_build": (
        c_int, [POINTER(VegasItem), c_int64, c_void_p, c_size_t, POINTER(VegasBatchInfo), c_void_p]),
    "tq_vegas_batch_phase": (
        c_int, [POINTER(VegasBatchInfo), c_void_p, c_int, c_void_p, c_double, c_double, c_uint64, c_void_p]),
    "tq_capture_while_begin": (c_int, [c_void_p, c_void_p, POINTER(c_uint64)]),
    "tq_capture_while_end": (c_int, [c_void_p]),
    "tq_vegas_warmup_fused": (c_int, [_VS, c_int, c_void_p, c_int64, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_update_map": (c_int, [_VS, c_double, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_smooth_weights": (c_int, [_VS, c_double, c_void_p, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_get_nh": (c_int, [_VS, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_get_nh_split": (c_int, [_VS, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_iterate_fused": (c_int, [_VS, c_int, c_void_p, c_int, c_int64, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_finish_iteration": (c_int, [_VS, c_double, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_finish_update_map": (c_int, [_VS, c_double, c_double, c_void_p, c_size_t, c_void_p]),
    "tq_vegas_strat_points": (c_int, [_VS, c_void_p, c_int64, c_void_p, c_void_p]),
    "tq_vegas_map_points": (c_int, [_VS, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "tq_vegas_accumulate": (
        c_int, [_VS, c_void_p, c_void_p, c_int64, c_int, c_int, c_void_p, c_size_t, c_void_p]),
    "tq_fp32_fma_probe": (c_int, [c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "tq_fp64_fma_probe": (c_int, [c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "tq_mc_fused": (
        c_int,
        [c_int, c_int, c_int64, c_void_p, c_int, c_void_p, c_uint64, c_uint64, c_uint64,
         c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
}

_lock = threading.Lock()
_lib = None

# Kernel launches issued through this binding (benchmark bookkeeping).
launches = [0]


def count_launches(n: int = 1) -> None:
    launches[0] += n


class TorchquadGB300Error(RuntimeError):
    """A kernel entry point returned a non-zero status."""

    def __init__(self, status: int, where: str):
        self.status = status
        msg = f"{where}: {status_string(status)} (status {status})"
        if status == TQ_ERR_CUDA:
            msg += f", cudaError {lib().tq_last_cuda_error()}"
        super().__init__(msg)


def load(path=None):
    """Load the shared library and declare every exported signature."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = str(path or lib_path())
        try:
            handle = ctypes.CDLL(p)
        except OSError as e:
            raise RuntimeError(
                f"torchquad_gb300 CUDA library not loadable at {p} ({e}). "
                "Build it with `python -m torchquad_gb300.build`; there is no CPU fallback."
            ) from None
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = handle
        return handle


def lib():
    return _lib if _lib is not None else load()


def status_string(status: int) -> str:
    return lib().tq_status_string(status).decode()


def check(status: int, where: str) -> None:
    if status != TQ_OK:
        raise TorchquadGB300Error(status, where)


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError(
            "torchquad_gb300 runs its integration kernels on a CUDA device only "
            "and no CUDA device is available (there is no CPU fallback)."
        )
    lib()
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


def body_stream(device, avoid=()) -> torch.cuda.Stream:
    """A stream for the body of a conditional node captured from the current
    stream.  torch hands out streams from a small per-device pool in turn,
    so a new stream can be the very stream being captured; another one is
    taken then (the body must be captured on a stream of its own).  Streams
    in `avoid` (torch streams) are skipped too."""
    taken = {torch.cuda.current_stream(device).cuda_stream} | {a.cuda_stream for a in avoid}
    for _ in range(64):
        s = torch.cuda.Stream(device=device)
        if s.cuda_stream not in taken:
            return s
    raise RuntimeError("no CUDA stream distinct from the capturing stream")


def dtype_code(dtype: torch.dtype) -> int:
    if dtype == torch.float32:
        return TQ_F32
    if dtype == torch.float64:
        return TQ_F64
    raise TypeError(f"unsupported dtype {dtype}; float32 and float64 are supported")


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


class _Workspace:
    """Per-device, per-stream grow-only scratch buffers owned by torch."""

    def __init__(self):
        self._bufs = {}

    def get(self, nbytes: int, slot: str = "main") -> torch.Tensor:
        dev = torch.cuda.current_device()
        key = (dev, torch.cuda.current_stream().cuda_stream, slot)
        buf = self._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            # tickets in the first 16 bytes must start at zero
            buf = torch.zeros(max(int(nbytes), 4096), dtype=torch.uint8, device=f"cuda:{dev}")
            self._bufs[key] = buf
        return buf


workspace = _Workspace()
