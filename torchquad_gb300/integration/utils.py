"""Host-side helpers: integration-domain set-up and checks.

Mirrors reference torchquad ``integration/utils.py`` behaviour for the torch
backend (``_setup_integration_domain`` :110-159, ``_check_integration_domain``
:162-206) with one difference by design: the domain tensor is placed on the
current CUDA device, where every kernel of this package runs.
"""
from __future__ import annotations

import warnings
import weakref

import torch

from .. import _lib as L
from ..utils.set_up_backend import _get_default_backend


def _check_backend(backend):
    if backend not in (None, "torch"):
        raise ValueError(
            f"Unsupported numerical backend: {backend}. torchquad_gb300 implements the "
            "torch backend only."
        )


def _host_domain_check(domain_list):
    """The list branch of _check_integration_domain (utils.py:171-191)."""
    dim = len(domain_list)
    if dim < 1:
        raise ValueError("len(integration_domain) needs to be 1 or larger.")
    for bounds in domain_list:
        if len(bounds) != 2:
            raise ValueError(bounds, " in ", domain_list, " does not specify a valid integration bound.")
        if bounds[0] > bounds[1]:
            raise ValueError(bounds, " in ", domain_list, " does not specify a valid integration bound.")
    return dim


def _check_integration_domain(integration_domain):
    """Validate a domain and return its dimension (utils.py:162-206)."""
    if not isinstance(integration_domain, torch.Tensor):
        return _host_domain_check(integration_domain)
    if integration_domain.dim() != 2:
        raise ValueError("The integration_domain tensor has an invalid shape")
    dim, num_bounds = integration_domain.shape
    if dim < 1:
        raise ValueError("integration_domain.shape[0] needs to be 1 or larger.")
    if num_bounds != 2:
        raise ValueError("integration_domain must have 2 values per boundary")
    if torch.jit.is_tracing():
        return dim
    if _validated(integration_domain):
        return dim
    if torch.min(integration_domain[:, 1] - integration_domain[:, 0]) < 0.0:
        raise ValueError("integration_domain has invalid boundary values")
    _remember_valid(integration_domain)
    return dim


# Device tensors already found valid, by identity, with the autograd version
# counter (bumped by every in-place write) and the storage address at the
# time: the check of a device tensor reads its values back (a device
# synchronisation), so an unchanged tensor is not checked again.
_VALID = {}


def _validated(t):
    e = _VALID.get(id(t))
    return e is not None and e[0]() is t and e[1] == t._version and e[2] == t.data_ptr()


def _remember_valid(t):
    if t.device.type != "cuda":
        return
    key = id(t)
    try:
        ref = weakref.ref(t, lambda _r, k=key: _VALID.pop(k, None))
    except TypeError:
        return
    _VALID[key] = (ref, t._version, t.data_ptr())


def _setup_integration_domain(dim, integration_domain, backend):
    """Return the domain as a [dim, 2] CUDA tensor (utils.py:110-159).

    A list (or None, meaning [-1, 1]^dim) becomes a tensor of torch's default
    dtype; a tensor keeps its dtype (integer domains become float64, as
    integration_grid.py:52-56 does) and is moved to the current CUDA device.
    """
    _check_backend(backend)
    if backend is None:
        _check_backend(_get_default_backend())
    device = L.require_cuda()
    if integration_domain is None:
        integration_domain = [[-1.0, 1.0]] * dim
    if not isinstance(integration_domain, torch.Tensor):
        if hasattr(integration_domain, "__array__") and not isinstance(integration_domain, (list, tuple)):
            integration_domain = integration_domain.tolist()
        values = [[float(b) for b in bounds] for bounds in integration_domain]
        t = torch.tensor(values, dtype=torch.get_default_dtype())
        if t.shape != (dim, 2):
            raise ValueError(
                "The integration domain has an unexpected shape. "
                f"Expected {(dim, 2)}, got {tuple(t.shape)}"
            )
        return t.to(device, non_blocking=True)
    t = integration_domain
    if not t.is_floating_point() or t.is_complex():
        t = t.to(torch.float64)
    if t.device != device:
        t = t.to(device)
    if tuple(t.shape) != (dim, 2):
        raise ValueError(
            "The integration domain has an unexpected shape. "
            f"Expected {(dim, 2)}, got {tuple(t.shape)}"
        )
    return t


def _host_domain_values(dim, integration_domain, backend):
    """For a domain given as host values (None, a list, a tuple or an array),
    the [dim][2] bounds as floats, with the checks of
    _setup_integration_domain; None for a tensor domain.  Lets a fused
    kernel take the bounds as launch arguments instead of a device copy."""
    if isinstance(integration_domain, torch.Tensor):
        return None
    _check_backend(backend)
    if backend is None:
        _check_backend(_get_default_backend())
    if integration_domain is None:
        return [(-1.0, 1.0)] * dim
    if hasattr(integration_domain, "__array__") and not isinstance(integration_domain, (list, tuple)):
        integration_domain = integration_domain.tolist()
    values = [(float(b[0]), float(b[1])) if len(b) == 2 else tuple(b) for b in integration_domain]
    if len(values) != dim or any(len(v) != 2 for v in values):
        raise ValueError(
            "The integration domain has an unexpected shape. "
            f"Expected {(dim, 2)}, got ({len(values)}, ...)"
        )
    return values


def _is_host_list(domain):
    return domain is None or not isinstance(domain, torch.Tensor)


def _warn_1d_result():
    warnings.warn(
        "DEPRECATION WARNING: In future versions of torchquad, an array-like object will be returned."
    )


def _split_integrand_values(values):
    """[N, *S] (real or complex) -> ([N, S_real] fp view, shape info)."""
    shape = tuple(values.shape[1:])
    is_complex = values.is_complex()
    v = values
    if is_complex:
        v = torch.view_as_real(v.contiguous())
    v = v.reshape(values.shape[0], -1)
    if v.dtype not in (torch.float32, torch.float64):
        v = v.to(torch.float64)
    return v.contiguous(), shape, is_complex


def _assemble_result(flat, shape, is_complex):
    if is_complex:
        flat = torch.view_as_complex(flat.reshape(-1, 2).contiguous())
    out = flat.reshape(shape) if len(shape) else flat.reshape(())
    is_1d = len(shape) == 0 or (len(shape) == 1 and shape[0] == 1)
    if is_1d:
        _warn_1d_result()
        out = out.squeeze()
    return out
