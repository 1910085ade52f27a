"""Thin typed wrappers over the C ABI used by the integrators.

Every function launches on torch's current CUDA stream and returns without
synchronising.  Scratch memory comes from a per-stream torch-owned workspace.
"""
from __future__ import annotations

import os

import torch

from .. import _lib as L

# Budget for one materialised chunk of points + values (bytes).
_DEFAULT_BUDGET = int(os.environ.get("TORCHQUAD_GB300_CHUNK_BYTES", str(8 << 30)))
_budget = [_DEFAULT_BUDGET]


def set_materialise_budget(nbytes: int) -> None:
    """Upper bound of device memory one materialised chunk (points and
    integrand values) may take; integrands that need more are evaluated in
    several calls of at most this size."""
    _budget[0] = max(1 << 16, int(nbytes))


def chunk_points(total: int, dim: int, esize: int) -> int:
    per = dim * esize + 2 * esize
    return max(1, min(total, _budget[0] // per))


def grid_points(rule, dim, n, domain, gl_nodes, start, count, dtype):
    pts = torch.empty((count, dim), dtype=dtype, device=domain.device)
    L.check(
        L.lib().tq_grid_points(
            L.dtype_code(domain.dtype), rule, dim, n, domain.data_ptr(), L.ptr(gl_nodes),
            start, count, pts.data_ptr(), L.stream_handle(),
        ),
        "tq_grid_points",
    )
    L.count_launches(1)
    return pts


def grid_weights(rule, dim, n, domain, gl_weights, start, count):
    w = torch.empty((count,), dtype=torch.float64, device=domain.device)
    L.check(
        L.lib().tq_grid_weights(
            L.dtype_code(domain.dtype), rule, dim, n, domain.data_ptr(), L.ptr(gl_weights),
            start, count, w.data_ptr(), L.stream_handle(),
        ),
        "tq_grid_weights",
    )
    L.count_launches(1)
    return w


def weighted_sum_into(acc, rule, dim, n, domain, gl_weights, start, values2d):
    """acc[2S] += sum_i w_i values2d[i, :] (compensated fp64)."""
    count, S = values2d.shape
    ws_bytes = L.lib().tq_weighted_sum_workspace_size(count, S)
    ws = L.workspace.get(ws_bytes, "wsum")
    L.check(
        L.lib().tq_weighted_sum(
            L.dtype_code(domain.dtype), rule, dim, n, domain.data_ptr(), L.ptr(gl_weights),
            start, count, values2d.data_ptr(), L.dtype_code(values2d.dtype), S,
            acc.data_ptr(), ws.data_ptr(), ws.numel(), L.stream_handle(),
        ),
        "tq_weighted_sum",
    )
    L.count_launches(1)


def finalize(acc, rule, dim, domain, n_points, S, out_dtype):
    out = torch.empty((S,), dtype=out_dtype, device=domain.device)
    L.check(
        L.lib().tq_finalize_sum(
            L.dtype_code(domain.dtype), rule, dim, domain.data_ptr(), n_points, acc.data_ptr(), S,
            out.data_ptr(), L.dtype_code(out_dtype), L.stream_handle(),
        ),
        "tq_finalize_sum",
    )
    L.count_launches(1)
    return out


class WeightedSum(torch.autograd.Function):
    """sum_i w_i * values[i, :] over a node range, differentiable in values.

    Forward runs tq_weighted_sum; backward materialises w_i with
    tq_grid_weights (ones for Monte Carlo) and returns grad * w_i."""

    @staticmethod
    def forward(ctx, values2d, rule, dim, n, domain, gl_weights, start):
        S = values2d.shape[1]
        acc = torch.zeros((2 * S,), dtype=torch.float64, device=values2d.device)
        weighted_sum_into(acc, rule, dim, n, domain, gl_weights, start, values2d)
        out = finalize(acc, L.TQ_RULE_TRAPEZOID, dim, domain, 1, S, values2d.dtype)
        ctx.meta = (rule, dim, n, domain, gl_weights, start, values2d.shape[0], values2d.dtype)
        return out

    @staticmethod
    def backward(ctx, grad):
        rule, dim, n, domain, gl_weights, start, count, dtype = ctx.meta
        if rule == L.TQ_RULE_MC:
            w = torch.ones((count,), dtype=torch.float64, device=grad.device)
        else:
            w = grid_weights(rule, dim, n, domain, gl_weights, start, count)
        g = (w[:, None] * grad.to(torch.float64)[None, :]).to(dtype)
        return g, None, None, None, None, None, None


def grid_fused(rule, dim, n, domain, gl_nodes, gl_weights, integrand, out_dtype):
    out = torch.empty((), dtype=out_dtype, device=domain.device)
    params = integrand.device_params(domain.device)
    ws = L.workspace.get(L.lib().tq_grid_fused_workspace_size(rule, dim, n), "fused")
    L.check(
        L.lib().tq_grid_fused(
            L.dtype_code(domain.dtype), rule, dim, n, domain.data_ptr(), L.ptr(gl_nodes),
            L.ptr(gl_weights), integrand.family, params.data_ptr(), out.data_ptr(),
            L.dtype_code(out_dtype), None, ws.data_ptr(), ws.numel(), L.stream_handle(),
        ),
        "tq_grid_fused",
    )
    L.count_launches(1)
    return out


def uniform(seed, stream_id, offset, size, dtype, device):
    out = torch.empty(size, dtype=dtype, device=device)
    L.check(
        L.lib().tq_uniform(
            L.dtype_code(dtype), seed, stream_id, offset, out.numel(), out.data_ptr(),
            L.stream_handle(),
        ),
        "tq_uniform",
    )
    L.count_launches(1)
    return out


def mc_fused(dim, n_points, domain, integrand, seed, stream_id, offset):
    out = torch.empty((), dtype=domain.dtype, device=domain.device)
    params = integrand.device_params(domain.device)
    ws = L.workspace.get(L.lib().tq_mc_fused_workspace_size(dim, n_points), "fused")
    L.check(
        L.lib().tq_mc_fused(
            L.dtype_code(domain.dtype), dim, n_points, domain.data_ptr(), integrand.family,
            params.data_ptr(), seed, stream_id, offset, out.data_ptr(), None, ws.data_ptr(),
            ws.numel(), L.stream_handle(),
        ),
        "tq_mc_fused",
    )
    L.count_launches(1)
    return out


def grid_adjoint(rule, dim, n, domain, gl_nodes, gl_weights, integrand):
    """(value, d/d domain [dim, 2], d/d params [2+2dim]) in fp64."""
    dev = domain.device
    val = torch.empty((), dtype=torch.float64, device=dev)
    gdom = torch.empty((dim, 2), dtype=torch.float64, device=dev)
    gpar = torch.empty((2 + 2 * dim,), dtype=torch.float64, device=dev)
    params = integrand.device_params(dev)
    ws = L.workspace.get(L.lib().tq_grid_adjoint_workspace_size(dim, n**dim), "adjoint")
    L.check(
        L.lib().tq_grid_adjoint(
            L.dtype_code(domain.dtype), rule, dim, n, domain.data_ptr(), L.ptr(gl_nodes),
            L.ptr(gl_weights), integrand.family, params.data_ptr(), val.data_ptr(), gdom.data_ptr(),
            gpar.data_ptr(), ws.data_ptr(), ws.numel(), L.stream_handle(),
        ),
        "tq_grid_adjoint",
    )
    L.count_launches(1)
    return val, gdom, gpar
