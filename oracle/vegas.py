"""VEGAS+ restated in numpy from the reference (test infrastructure only).

Follows torchquad v0.5.0 vegas_map.py (VEGASMap :9-261), vegas_stratification.py
(VEGASStratification :7-165) and vegas.py (VEGAS :13-362) operation by
operation in the working dtype ``dt`` (np.float32 / np.float64).  The
scatter-adds of utils.py:61-76 (torch's scatter_add_ on the CPU: one add
per point, in point order, rounded to dt each time) are np.add.at, which
adds the same way.  Uniform numbers come from an injected stream with
``uniform(size, dtype)``.

Test infrastructure only: the library never imports this module.
"""
from __future__ import annotations

import math
import warnings

import numpy as np

from .grid import linspace



def _sum_lr(xs, zero=0.0):
    t = zero
    for x in xs:
        t = t + x
    return t


class Map:
    """vegas_map.py:9-261."""

    def __init__(self, B, dim, dt, alpha=0.5):
        self.B, self.dim, self.dt, self.alpha = B, dim, dt, alpha
        self.dx_edges = (np.ones((dim, B), dtype=dt) / dt(B)).astype(dt)  # :34-37
        self.x_edges = np.repeat(linspace(0.0, 1.0, B + 1, dt)[None, :], dim, axis=0)  # :38-39
        self.reset_weight()

    def reset_weight(self):  # :174-183
        self.weights = np.zeros((self.dim, self.B), dtype=self.dt)
        self.counts = np.zeros((self.dim, self.B), dtype=np.int64)

    def interval_id(self, y):  # :76-85
        return np.floor(y * self.dt(self.B)).astype(np.int64)

    def interval_offset(self, y):  # :87-97
        yB = (y * self.dt(self.B)).astype(self.dt)
        return (yB - np.floor(yB)).astype(self.dt)

    def get_X(self, y):  # :44-58
        ID, off = self.interval_id(y), self.interval_offset(y)
        res = np.zeros_like(y)
        for i in range(self.dim):
            res[:, i] = self.x_edges[i, ID[:, i]] + (self.dx_edges[i, ID[:, i]] * off[:, i]).astype(self.dt)
        return res

    def get_Jac(self, y):  # :60-74
        ID = self.interval_id(y)
        jac = np.ones(y.shape[0], dtype=y.dtype)
        for i in range(self.dim):
            jac = (jac * (self.dt(self.B) * self.dx_edges[i, ID[:, i]]).astype(self.dt)).astype(self.dt)
        return jac

    def accumulate_weight(self, y, jf2):  # :99-111
        ID = self.interval_id(y)
        jf2 = np.asarray(jf2, dtype=self.dt)
        for i in range(self.dim):
            np.add.at(self.weights[i], ID[:, i], jf2)
            self.counts[i] += np.bincount(ID[:, i], minlength=self.B)

    @staticmethod
    def smooth_map(weights, counts, alpha):  # :113-172
        dt = weights.dtype.type
        weights = weights.copy()
        z = counts == 0
        if np.any(z):
            nz = ~z
            weights[nz] = (weights[nz] / counts[nz].astype(dt)).astype(dt)
            for _ in range(10):
                weights[:, :-1] = np.where(z[:, :-1], weights[:, 1:], weights[:, :-1])
                z[:, :-1] = z[:, :-1] & z[:, 1:]
                weights[:, 1:] = np.where(z[:, 1:], weights[:, :-1], weights[:, 1:])
                z[:, 1:] = z[:, 1:] & z[:, :-1]
                if not np.any(z):
                    break
        else:
            weights = (weights / counts.astype(dt)).astype(dt)
        dim, B = weights.shape
        sums = weights.astype(np.float64).sum(axis=1).astype(dt).reshape(dim, 1)
        if np.any(sums == 0.0):
            return None
        i = B - 2
        d = np.concatenate(
            [
                (dt(7.0) * weights[:, 0:1]).astype(dt) + weights[:, 1:2],
                (weights[:, :-2] + (dt(6.0) * weights[:, 1:-1]).astype(dt)).astype(dt) + weights[:, 2:],
                weights[:, i : i + 1] + (dt(7.0) * weights[:, i + 1 : i + 2]).astype(dt),
            ],
            axis=1,
        ).astype(dt)
        d = (d / (dt(8.0) * sums).astype(dt)).astype(dt)
        nz = d != 0
        with np.errstate(divide="ignore", invalid="ignore"):
            t = ((d[nz] - dt(1.0)) / np.log(d[nz])).astype(dt)
            d[nz] = np.sqrt(t) if alpha == 0.5 else np.power(t, dt(alpha))
        return d.astype(dt)

    def update_map(self):  # :185-261
        dt = self.dt
        sw = self.smooth_map(self.weights, self.counts, self.alpha)
        if sw is None:
            warnings.warn("Cannot update the VEGASMap.", RuntimeWarning)
            self.reset_weight()
            return False
        delta_w = (sw.astype(np.float64).sum(axis=1).astype(dt) / dt(self.B)).astype(dt)
        B = self.B
        for i in range(self.dim):
            delta = delta_w[i]
            mult = (np.cumsum(sw[i, :-1].astype(np.float64)) / np.float64(delta)).astype(np.int64)
            num = np.bincount(mult, minlength=B + 1)[: B + 1].astype(np.int64)
            val = np.zeros(B + 1, dtype=dt)
            for j, m in enumerate(mult):  # sequential scatter in dt, as torch CPU does
                val[m] = dt(val[m] + sw[i, j])
            indices = np.cumsum(num[:-2])
            d_accu = np.cumsum((delta - val[:-2]).astype(dt).astype(np.float64)).astype(dt)
            new = (self.x_edges[i][indices]
                   + ((d_accu / sw[i][indices]).astype(dt) * self.dx_edges[i][indices]).astype(dt)).astype(dt)
            self.x_edges[i][1:-1] = new
            fin = np.isfinite(self.x_edges[i])
            if not np.all(fin):
                mid = (dt(0.5) * (self.x_edges[i][:-2] + self.x_edges[i][2:])).astype(dt)
                self.x_edges[i][1:-1] = np.where(fin[1:-1], self.x_edges[i][1:-1], mid)
                if not np.all(np.isfinite(self.x_edges[i])):
                    raise RuntimeError("Could not replace all infinite edges")
            self.dx_edges[i] = (self.x_edges[i][1:] - self.x_edges[i][:-1]).astype(dt)
        self.reset_weight()
        return True


class Strat:
    """vegas_stratification.py:7-165."""

    def __init__(self, N_increment, dim, dt, beta=0.75):
        self.dim, self.dt, self.beta = dim, dt, beta
        n = int((N_increment / 4.0) ** (1.0 / dim))
        self.N_strat = max(1, 1000 if n > 1000 else n)
        self.N_cubes = self.N_strat**dim
        self.V_cubes = (1.0 / self.N_strat) ** dim
        self.JF = np.zeros(self.N_cubes, dtype=dt)
        self.JF2 = np.zeros(self.N_cubes, dtype=dt)
        self.dh = (np.ones(self.N_cubes, dtype=dt) * dt(1.0) / dt(self.N_cubes)).astype(dt)
        self.strat_counts = np.zeros(self.N_cubes, dtype=dt)

    def get_NH(self, nevals_exp):  # :92-103
        nh = np.floor((self.dh * self.dt(nevals_exp)).astype(self.dt))
        return np.clip(nh, 2, None).astype(np.int64)

    def positions(self):  # :105-138
        idx = np.arange(self.N_cubes, dtype=np.int64)
        strides = self.N_strat ** np.arange(self.dim, dtype=np.int64)
        p = idx[:, None] // strides[None, :]
        p[:, :-1] = p[:, :-1] - self.N_strat * p[:, 1:]
        return p

    def get_Y(self, nevals, u):  # :140-165 with the uniforms given
        pos = np.repeat(self.positions(), nevals, axis=0).astype(self.dt)
        y = ((pos + u).astype(self.dt) / self.dt(self.N_strat)).astype(self.dt)
        y[y >= 1.0] = self.dt(0.999999)
        return y

    def accumulate_weight(self, nevals, w):  # :46-70
        idx = np.repeat(np.arange(self.N_cubes), nevals)
        w = np.asarray(w, dtype=self.dt)
        self.JF = np.zeros(self.N_cubes, dtype=self.dt)
        self.JF2 = np.zeros(self.N_cubes, dtype=self.dt)
        np.add.at(self.JF, idx, w)
        np.add.at(self.JF2, idx, (w * w).astype(self.dt))
        self.strat_counts = nevals.astype(self.dt)
        return self.JF, self.JF2

    def update_DH(self):  # :72-90
        dt = self.dt
        V, V2 = dt(self.V_cubes), dt(self.V_cubes * self.V_cubes)
        q = ((V * self.JF).astype(dt) / self.strat_counts).astype(dt)
        d = (((V2 * self.JF2).astype(dt) / self.strat_counts).astype(dt) - (q * q).astype(dt)).astype(dt)
        d[d < 0.0] = 0.0
        self.dh = np.power(d, dt(self.beta)).astype(dt)
        s = dt(self.dh.astype(np.float64).sum())
        if s != 0:
            self.dh = (self.dh / s).astype(dt)


class Vegas:
    """vegas.py:13-362 with an injected uniform stream; fn(x) -> f on [N, dim]."""

    def integrate(self, fn, dim, N, domain, rng, dt=np.float32, n_intervals=None,
                  use_grid_improve=True, eps_rel=0, eps_abs=0, max_iterations=20, use_warmup=True,
                  record=None):
        domain = np.asarray(domain, dtype=dt)
        self.dim, self.dt, self.N = dim, dt, N
        self.rng = rng
        self.max_iterations, self.eps_rel, self.eps_abs = max_iterations, eps_rel, eps_abs
        self.fevals = 0
        self.starting_N = N // (max_iterations + 5)
        self.N_increment = N // (max_iterations + 5)
        starts = domain[:, 0]
        sizes = (domain[:, 1] - starts).astype(dt)
        vol = dt(np.prod(sizes))
        self.fn = lambda x: (fn((x * sizes).astype(dt) + starts) * vol).astype(dt)
        B = n_intervals if n_intervals is not None else max(2, self.N_increment // 10)
        self.map = Map(B, dim, dt)
        self.strat = Strat(self.N_increment, dim, dt)
        self.results, self.sigma2, self.it = [], [], 0
        self.record = record
        if use_warmup:
            self.warmup(5, self.starting_N // 5)
        while True:
            self.it += 1
            self.results.append(0.0)
            self.sigma2.append(0.0)
            self.run_iteration(use_grid_improve)
            if self.check_abort():
                break
        return self.get_result()

    def warmup(self, n_it, ns):  # :211-266
        for _ in range(n_it):
            y = (self.rng.uniform([ns, self.dim], self.dt) * self.dt(0.999999)).astype(self.dt)
            x = self.map.get_X(y)
            f = self.fn(x)
            self.fevals += ns
            jf = (f * self.map.get_Jac(y)).astype(self.dt)
            self.map.accumulate_weight(y, (jf * jf).astype(self.dt))
            self.map.update_map()

    def run_iteration(self, use_grid_improve):  # :268-315
        dt = self.dt
        rec = {} if self.record is not None else None
        if rec is not None:
            rec.update(x_edges=self.map.x_edges.copy(), dx_edges=self.map.dx_edges.copy(), dh=self.strat.dh.copy())
        neval = self.strat.get_NH(self.starting_N)
        M = int(neval.sum())
        u = self.rng.uniform([M, self.dim], dt)
        y = self.strat.get_Y(neval, u)
        x = self.map.get_X(y)
        f = self.fn(x)
        self.fevals += M
        jac = self.map.get_Jac(y)
        jf = (f * jac).astype(dt)
        if use_grid_improve:
            self.map.accumulate_weight(y, (jf * jf).astype(dt))
        JF, JF2 = self.strat.accumulate_weight(neval, jf)
        n = neval.astype(np.float64)
        V = self.strat.V_cubes
        ih = JF.astype(np.float64) * (V / n)
        sig2 = np.abs(JF2.astype(np.float64) / n * (V * V) - ih * ih)
        self.results[-1] = float(ih.sum())
        self.sigma2[-1] = float((sig2 / n).sum())
        if rec is not None:
            rec.update(neval=neval.copy(), M=M, counts=self.map.counts.copy(), weights=self.map.weights.copy(),
                       JF=JF.copy(), JF2=JF2.copy(), result=self.results[-1], sigma2=self.sigma2[-1],
                       y_head=y[:64].copy())
        if use_grid_improve:
            self.map.update_map()
        self.strat.update_DH()
        if rec is not None:
            rec.update(x_edges_new=self.map.x_edges.copy(), dh_new=self.strat.dh.copy())
            self.record.append(rec)

    # The reference keeps results and variances as 0-d tensors of the
    # working dtype: the abort test and the estimate below round every
    # operation to dt (numpy scalars), Python scalar operands rounded to dt
    # first; sums run left to right from zero (Python's builtin sum of
    # floats is compensated since 3.12); x / 0 gives inf or nan.
    def check_abort(self):  # :161-209
        if self.it % 5 > 0:
            return False
        dt = self.dt
        with np.errstate(all="ignore"):
            res_abs = abs(self.get_result())
            err = self.get_error()
            q = self.get_chisq() / dt(5.0)
            if (err <= dt(self.eps_rel) * res_abs or err <= dt(self.eps_abs)) and q < 1.0:
                return True
            if q < 1.0:
                if res_abs == 0.0:
                    self.starting_N += self.N_increment
                else:
                    acc = err / res_abs
                    x = dt(self.starting_N) * np.sqrt(acc / dt(self.eps_rel + 1e-8))
                    self.starting_N = min(self.starting_N + self.N_increment, int(x))
            elif q > 1.0:
                self.starting_N += self.N_increment
        if self.fevals + self.starting_N * 5 > self.N:
            return True
        if self.it + 5 > self.max_iterations:
            return True
        self.results, self.sigma2 = [], []
        return False

    def _rows(self):
        dt = self.dt
        return [dt(r) for r in self.results], [dt(s) for s in self.sigma2]

    def get_result(self):  # :318-335
        dt = self.dt
        rs, ss = self._rows()
        with np.errstate(all="ignore"):
            if any(s == 0.0 for s in ss):
                return _sum_lr(rs, dt(0)) / dt(len(rs))
            return _sum_lr((r / s for r, s in zip(rs, ss)), dt(0)) / _sum_lr((dt(1) / s for s in ss), dt(0))

    def get_error(self):  # :337-346
        dt = self.dt
        _, ss = self._rows()
        with np.errstate(all="ignore"):
            res = _sum_lr((dt(1) / s for s in ss if s != 0.0), dt(0))
            return ss[0] if res == 0 else dt(1) / np.sqrt(res)

    def get_chisq(self):  # :348-362
        dt = self.dt
        I = self.get_result()
        rs, ss = self._rows()
        with np.errstate(all="ignore"):
            return _sum_lr(((r - I) * (r - I) / s for r, s in zip(rs, ss) if r != I), dt(0))
