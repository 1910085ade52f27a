"""Gradient of the tensor-product rules (test infrastructure only).

The reference differentiates a grid rule through torch autograd over its
materialised grid: nodes x_k = a_k + t_k (b_k - a_k) (integration_grid.py:
74-88, utils.py:36-52 _linspace_with_grads; gaussian.py:81-84,159-162 for
Gauss-Legendre), weights proportional to prod_k (b_k - a_k)
(trapezoid.py:27-37, simpson.py:29-46, boole.py:29-48, gaussian.py:131-144).
This restates the gradient of that discrete rule in numpy (fp64) for the
built-in separable families f = c F(sum_k g_k(x_k)):

    I        = sum_i W_i f(x_i)
    dI/db_k  =  I / L_k + sum_i W_i df/dx_k (x_i) t_ik
    dI/da_k  = -I / L_k + sum_i W_i df/dx_k (x_i) (1 - t_ik)
    dI/dp    = sum_i W_i df/dp (x_i)

It is the CPU baseline of the differentiation workload and a CPU check of
the adjoint kernels on small grids.
"""
import math

import numpy as np

from .grid import GAUSS, BOOLE, SIMPSON, TRAPEZOID, linspace
from .integrands import EXP_SUM, GAUSSIAN, OSCILLATORY, SUM_SIN


def _unit_rule(rule, n):
    """Unit nodes t in [0, 1] and 1-D weights per unit length."""
    if rule == GAUSS:
        r, w = np.polynomial.legendre.leggauss(n)
        return (r + 1.0) * 0.5, w * 0.5
    t = linspace(0.0, 1.0, n, np.float64)
    h = 1.0 / (n - 1)
    if rule == TRAPEZOID:
        c = np.full(n, 2.0)
        c[[0, -1]] = 1.0
        return t, c * h / 2.0
    if rule == SIMPSON:
        c = np.where(np.arange(n) % 2 == 1, 4.0, 2.0)
        c[[0, -1]] = 1.0
        return t, c * h / 3.0
    m = np.arange(n) % 4
    c = np.where(m % 2 == 1, 32.0, np.where(m == 2, 12.0, 14.0))
    c[[0, -1]] = 7.0
    return t, c * h / 22.5


def value_and_grad(family, params, rule, dim, n, domain):
    """(I, dI/ddomain [dim, 2], dI/dparams [2 + 2 dim]) for the family with
    params [c, b, a_k, u_k] over the n^dim grid of the rule on domain."""
    domain = np.asarray(domain, dtype=np.float64)
    lo, hi = domain[:, 0], domain[:, 1]
    L = hi - lo
    c, b = float(params[0]), float(params[1])
    a = np.asarray(params[2:2 + dim], dtype=np.float64)
    u = np.asarray(params[2 + dim:2 + 2 * dim], dtype=np.float64)
    t1, w1 = _unit_rule(rule, n)
    T = np.stack([m.ravel() for m in np.meshgrid(*([t1] * dim), indexing="ij")], axis=1)
    W = np.prod(np.stack([m.ravel() for m in np.meshgrid(*([w1] * dim), indexing="ij")], axis=1),
                axis=1) * np.prod(L)
    X = lo + T * L
    if family == GAUSSIAN:
        d = X - u
        s = (a * d * d).sum(1)
        F = np.exp(-s)
        Fp = -F
        gp, ga, gu = 2 * a * d, d * d, -2 * a * d
    elif family == SUM_SIN:
        s = np.sin(a * X).sum(1)
        F, Fp = s, np.ones_like(s)
        cs = np.cos(a * X)
        gp, ga, gu = a * cs, X * cs, np.zeros_like(X)
    else:
        s = (a * X).sum(1)
        if family == EXP_SUM:
            F = np.exp(s + b)
            Fp = F
        else:
            F = np.cos(2.0 * math.pi * b + s)
            Fp = -np.sin(2.0 * math.pi * b + s)
        gp, ga, gu = np.broadcast_to(a, X.shape), X, np.zeros_like(X)
    I = c * np.dot(W, F)
    wfp = c * W * Fp
    sx = wfp @ gp
    st = wfp @ (gp * T)
    gdom = np.stack([-I / L + (sx - st), I / L + st], axis=1)
    gpar = np.zeros(2 + 2 * dim)
    gpar[0] = np.dot(W, F)
    if family == EXP_SUM:
        gpar[1] = I
    elif family == OSCILLATORY:
        gpar[1] = 2.0 * math.pi * np.dot(W, c * Fp)
    gpar[2:2 + dim] = wfp @ ga
    gpar[2 + dim:] = wfp @ gu
    return I, gdom, gpar


__all__ = ["value_and_grad", "TRAPEZOID", "SIMPSON", "BOOLE", "GAUSS"]
