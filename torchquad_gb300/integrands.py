"""Built-in integrand families, evaluated inside the fused kernels.

Every family has the separable-sum form ``f(x) = F(sum_k g_k(x_k))`` with
parameters ``c, b, a_k, u_k`` (layout of the fp64 ``params`` array in
``include/torchquad_gb300.h``):

=================  =====================================  =========================
family             f(x)                                   used by
=================  =====================================  =========================
``ExpSum``         c * exp(sum_k a_k x_k + b)             plain Simpson, exp(x0+x1+x2)
``GaussianPeak``   c * exp(-sum_k a_k (x_k - u_k)^2)      VEGAS peak, batched Gaussians
``Oscillatory``    c * cos(2 pi b + sum_k a_k x_k)        differentiation
``SumSin``         c * sum_k sin(a_k x_k)                 5-D sum of sines
=================  =====================================  =========================

An instance is also an ordinary vectorised torch callable (``f(x)`` with
``x`` of shape ``[N, dim]``), so it works with every integrator, on the
materialised path, and as the integrand handed to the reference
implementation when checking parity.  Passing an instance to ``integrate``
selects the fused kernel, where no point tensor is materialised.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib as L


def _as_param(v, dim, name):
    if isinstance(v, torch.Tensor):
        if v.dim() == 0:
            v = v.reshape(1).expand(dim)
        if v.shape != (dim,):
            raise ValueError(f"{name} must have shape ({dim},), got {tuple(v.shape)}")
        return v
    if isinstance(v, (int, float)):
        return torch.full((dim,), float(v), dtype=torch.float64)
    t = torch.as_tensor(v, dtype=torch.float64)
    if t.shape != (dim,):
        raise ValueError(f"{name} must have shape ({dim},), got {tuple(t.shape)}")
    return t


def _as_scalar(v):
    return v if isinstance(v, torch.Tensor) else torch.tensor(float(v), dtype=torch.float64)


class BuiltinIntegrand:
    """Base class: a family id plus parameters ``c, b, a[dim], u[dim]``."""

    family = 0

    def __init__(self, dim, a=1.0, b=0.0, c=1.0, u=0.0):
        if dim < 1:
            raise ValueError("dim must be >= 1")
        self.dim = int(dim)
        self.a = _as_param(a, self.dim, "a")
        self.u = _as_param(u, self.dim, "u")
        self.b = _as_scalar(b)
        self.c = _as_scalar(c)
        self._dev_params = {}
        self._np_key = None
        self._np = None
        if not any(isinstance(v, torch.Tensor) for v in (a, u, b, c)):
            # plain numbers: the host vector without torch operations
            self._np = np.concatenate([[float(c), float(b)], self.a.numpy(), self.u.numpy()])
            self._np_key = self._params_key()

    # parameters that may carry gradients
    def parameters(self):
        return [self.c, self.b, self.a, self.u]

    def requires_grad(self) -> bool:
        return any(p.requires_grad for p in self.parameters())

    def params_vector(self) -> torch.Tensor:
        """fp64 ``[c, b, a_0..a_{d-1}, u_0..u_{d-1}]`` (detached, on the host)."""
        return torch.cat(
            [
                self.c.detach().reshape(1).to("cpu", torch.float64),
                self.b.detach().reshape(1).to("cpu", torch.float64),
                self.a.detach().to("cpu", torch.float64),
                self.u.detach().to("cpu", torch.float64),
            ]
        )

    def _params_key(self):
        # identity and autograd version counter (bumped by in-place writes)
        # of each parameter tensor
        return tuple((id(p), p._version) for p in (self.c, self.b, self.a, self.u))

    def params_numpy(self):
        """The parameter vector as a cached fp64 numpy array, refreshed when a
        parameter tensor is replaced or written in place."""
        key = self._params_key()
        if key != self._np_key:
            self._np = self.params_vector().numpy()
            self._np_key = key
        return self._np

    def device_params(self, device) -> torch.Tensor:
        """Cached device copy of the parameter vector (re-uploaded if changed)."""
        host = self.params_numpy()
        key = (str(device),)
        cached = self._dev_params.get(key)
        if cached is not None and cached[0] is host:
            return cached[1]
        dev = torch.from_numpy(host).to(device, non_blocking=False)
        self._dev_params[key] = (host, dev)
        return dev

    # ---- torch evaluation (same operation order as the device functions)
    def _term(self, k, xk, a, u):
        return a[k] * xk

    def _outer(self, s, c, b):
        raise NotImplementedError

    def __call__(self, x):
        if x.dim() != 2 or x.shape[1] != self.dim:
            raise ValueError(f"expected points of shape [N, {self.dim}], got {tuple(x.shape)}")
        dt, dev = x.dtype, x.device
        a = self.a.to(dev, dt)
        u = self.u.to(dev, dt)
        c = self.c.to(dev, dt)
        b = self.b.to(dev, dt)
        s = self._term(0, x[:, 0], a, u)
        for k in range(1, self.dim):
            s = s + self._term(k, x[:, k], a, u)
        return self._outer(s, c, b)

    def __repr__(self):
        return f"{type(self).__name__}(dim={self.dim})"

    def exact(self, domain) -> float:
        """The integral over the box domain [[lo, hi]] * dim in closed form
        (fp64 on the host): the reference value accuracy is reported
        against."""
        raise NotImplementedError

    def _box(self, domain):
        d = np.asarray(domain.detach().cpu() if isinstance(domain, torch.Tensor) else domain,
                       dtype=np.float64).reshape(self.dim, 2)
        p = self.params_numpy()
        return d[:, 0], d[:, 1], float(p[0]), float(p[1]), p[2:2 + self.dim], p[2 + self.dim:]


class ExpSum(BuiltinIntegrand):
    """f(x) = c * exp(sum_k a_k x_k + b)."""

    family = L.TQ_FN_EXP_SUM

    def __init__(self, dim, a=1.0, b=0.0, c=1.0):
        super().__init__(dim, a=a, b=b, c=c)

    def _outer(self, s, c, b):
        return c * torch.exp(s + b)

    def exact(self, domain):
        lo, hi, c, b, a, _ = self._box(domain)
        v = c * math.exp(b)
        for k in range(self.dim):
            v *= (hi[k] - lo[k]) if a[k] == 0.0 else (math.exp(a[k] * hi[k]) - math.exp(a[k] * lo[k])) / a[k]
        return v


class GaussianPeak(BuiltinIntegrand):
    """f(x) = c * exp(-sum_k a_k (x_k - u_k)^2)."""

    family = L.TQ_FN_GAUSSIAN

    def __init__(self, dim, a=1.0, u=0.5, c=1.0):
        super().__init__(dim, a=a, b=0.0, c=c, u=u)

    @classmethod
    def normal(cls, dim, mean=0.5, sigma=0.05):
        """Product of normal densities N(mean, sigma^2) in every dimension."""
        return cls(
            dim,
            a=1.0 / (2.0 * sigma * sigma),
            u=mean,
            c=(1.0 / (sigma * math.sqrt(2.0 * math.pi))) ** dim,
        )

    def _term(self, k, xk, a, u):
        d = xk - u[k]
        return a[k] * (d * d)

    def _outer(self, s, c, b):
        return c * torch.exp(-s)

    def exact(self, domain):
        lo, hi, c, _, a, u = self._box(domain)
        v = c
        for k in range(self.dim):
            r = math.sqrt(a[k])
            v *= math.sqrt(math.pi / a[k]) / 2.0 * (math.erf(r * (hi[k] - u[k])) - math.erf(r * (lo[k] - u[k])))
        return v


class Oscillatory(BuiltinIntegrand):
    """f(x) = c * cos(2 pi b + sum_k a_k x_k)   (b plays the role of u)."""

    family = L.TQ_FN_OSCILLATORY

    def __init__(self, dim, a=1.0, b=0.0, c=1.0):
        super().__init__(dim, a=a, b=b, c=c)

    def _outer(self, s, c, b):
        return c * torch.cos((2.0 * math.pi) * b + s)

    def exact(self, domain):
        # Re[c e^{i 2 pi b} prod_k (e^{i a_k hi_k} - e^{i a_k lo_k}) / (i a_k)]
        lo, hi, c, b, a, _ = self._box(domain)
        z = complex(math.cos(2.0 * math.pi * b), math.sin(2.0 * math.pi * b))
        for k in range(self.dim):
            if a[k] == 0.0:
                z *= hi[k] - lo[k]
            else:
                e1 = complex(math.cos(a[k] * hi[k]), math.sin(a[k] * hi[k]))
                e0 = complex(math.cos(a[k] * lo[k]), math.sin(a[k] * lo[k]))
                z *= (e1 - e0) / complex(0.0, a[k])
        return c * z.real


class SumSin(BuiltinIntegrand):
    """f(x) = c * sum_k sin(a_k x_k)."""

    family = L.TQ_FN_SUM_SIN

    def __init__(self, dim, a=1.0, c=1.0):
        super().__init__(dim, a=a, b=0.0, c=c)

    def _term(self, k, xk, a, u):
        return torch.sin(a[k] * xk)

    def _outer(self, s, c, b):
        return c * s

    def exact(self, domain):
        lo, hi, c, _, a, _ = self._box(domain)
        vol = float(np.prod(hi - lo))
        v = 0.0
        for k in range(self.dim):
            w = hi[k] - lo[k]
            ik = w if a[k] == 0.0 else (math.cos(a[k] * lo[k]) - math.cos(a[k] * hi[k])) / a[k]
            v += ik * vol / w if w != 0.0 else 0.0
        return c * v


__all__ = ["BuiltinIntegrand", "ExpSum", "GaussianPeak", "Oscillatory", "SumSin"]
