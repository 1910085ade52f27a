"""Tensor-product grid rules, restated from the reference:
nodes (integration_grid.py:28-103, utils.py:24-58 torch linspace),
composite rules collapsing one dimension at a time (trapezoid.py:27-37,
simpson.py:29-46, boole.py:29-48, gaussian.py:131-144), N adjustment
(simpson.py:53-83, boole.py:55-84)."""
import numpy as np

TRAPEZOID, SIMPSON, BOOLE, GAUSS = 0, 1, 2, 3


def _fma(x, y, z, dt):
    """x * y + z rounded once to dt (x, y, z arrays or scalars of dt): the
    product and sum are formed in extended precision first."""
    ld = np.longdouble
    return (np.asarray(x, dtype=ld) * np.asarray(y, dtype=ld) + np.asarray(z, dtype=ld)).astype(dt)


def linspace(a, b, n, dt):
    """torch CPU linspace: step in dt, first half fma(step, i, a), second
    half fma(-step, n-1-i, b)."""
    a, b = dt(a), dt(b)
    step = dt((b - a) / dt(n - 1))
    i = np.arange(n)
    lo = _fma(step, i[: n // 2].astype(dt), a, dt)
    hi = _fma(-step, (n - 1 - i[n // 2:]).astype(dt), b, dt)
    return np.concatenate([lo, hi]).astype(dt)


def n_per_dim(N, dim):
    return int(N ** (1.0 / dim) + 1e-8)


def adjust_N(rule, dim, N):
    n = n_per_dim(N, dim)
    if rule == SIMPSON:
        if n < 3:
            return 3**dim
        if n % 2 != 1:
            return (n - 1) ** dim
    if rule == BOOLE:
        if n < 5:
            return 5**dim
        if (n - 1) % 4 != 0:
            return (n - ((n - 1) % 4)) ** dim
    return N


def nodes_1d(rule, a, b, n, dt):
    if rule == GAUSS:
        r, _ = np.polynomial.legendre.leggauss(n)
        return ((dt(b) - dt(a)) / dt(2)).astype(np.float64) * r + ((dt(a) + dt(b)) / dt(2)).astype(np.float64)
    return linspace(a, b, n, dt)


def points(rule, domain, n, dt):
    dim = domain.shape[0]
    g = [nodes_1d(rule, domain[k, 0], domain[k, 1], n, dt) for k in range(dim)]
    mesh = np.meshgrid(*g, indexing="ij")
    return np.stack([m.ravel() for m in mesh], axis=1), np.array([x[1] - x[0] for x in g])


def apply_rule(rule, f, dim, hs, domain):
    """f shaped [n]*dim; collapse the last axis dim times."""
    for k in range(dim):
        h = hs[k]
        if rule == TRAPEZOID:
            f = h / 2.0 * (f[..., 0:-1] + f[..., 1:])
        elif rule == SIMPSON:
            f = h / 3.0 * (f[..., 0:-2][..., ::2] + 4 * f[..., 1:-1][..., ::2] + f[..., 2:][..., ::2])
        elif rule == BOOLE:
            f = h / 22.5 * (
                7 * f[..., 0:-4][..., ::4]
                + 32 * f[..., 1:-3][..., ::4]
                + 12 * f[..., 2:-2][..., ::4]
                + 32 * f[..., 3:-1][..., ::4]
                + 7 * f[..., 4:][..., ::4]
            )
        if rule == GAUSS:
            f = 0.5 * (domain[k][1] - domain[k][0]) * np.sum(f, axis=-1)
        else:
            f = np.sum(f, axis=-1)
    return f


def integrate(fn, rule, dim, N, domain, dt=np.float64):
    """fn(x [M, dim]) -> [M]; returns the reference's quadrature value."""
    domain = np.asarray(domain, dtype=dt)
    N = adjust_N(rule, dim, N)
    n = n_per_dim(N, dim)
    pts, hs = points(rule, domain, n, dt)
    f = fn(pts)
    if rule == GAUSS:
        _, w = np.polynomial.legendre.leggauss(n)
        W = np.prod(np.stack(np.meshgrid(*([w] * dim), indexing="ij")), axis=0).ravel()
        f = f * W
    return apply_rule(rule, f.reshape([n] * dim), dim, hs, domain)
