"""numpy evaluation of the built-in integrand families (same operation
order as torchquad_gb300.integrands and the device functions)."""
import math

import numpy as np

EXP_SUM, GAUSSIAN, OSCILLATORY, SUM_SIN = 1, 2, 3, 4


def evaluate(family, params, x):
    """params = [c, b, a_0..a_{d-1}, u_0..u_{d-1}] (fp64); x [N, d]."""
    dt = x.dtype.type
    d = x.shape[1]
    c, b = dt(params[0]), dt(params[1])
    a = params[2 : 2 + d].astype(x.dtype)
    u = params[2 + d : 2 + 2 * d].astype(x.dtype)

    def term(k):
        if family == GAUSSIAN:
            t = x[:, k] - u[k]
            return a[k] * (t * t)
        if family == SUM_SIN:
            return np.sin(a[k] * x[:, k])
        return a[k] * x[:, k]

    s = term(0)
    for k in range(1, d):
        s = s + term(k)
    if family == EXP_SUM:
        return c * np.exp(s + b)
    if family == GAUSSIAN:
        return c * np.exp(-s)
    if family == OSCILLATORY:
        return c * np.cos(dt(2.0 * math.pi) * b + s)
    return c * s
