"""Monte Carlo (monte_carlo.py:20-106) on injected uniforms."""
import numpy as np


def integrate(fn, dim, N, domain, uniforms):
    """uniforms [N, dim] in [0, 1); x = u * (b - a) + a; V * sum f / N."""
    domain = np.asarray(domain)
    dt = uniforms.dtype.type
    a = domain[:, 0].astype(dt)
    w = (domain[:, 1] - domain[:, 0]).astype(dt)
    x = uniforms * w + a
    f = fn(x)
    vol = np.prod(w)
    return vol * np.sum(f, axis=0) / N
