"""Time the unmodified reference torchquad's per-call CPU path on the
workloads the GPU build batches, differentiates and serves.

Run in a container where the reference source is present:

    python tests/golden/time_reference.py /root/reference [--budget 20]

The reference (with the dispatch-only stand-ins of ``tests/golden/refshim``
for autoray and loguru) runs on torch CPU with every host thread; each
workload is the loop of per-call ``integrate`` calls a reference user runs,
over the same seeded inputs as ``bench.py``, in order, until the time budget
is spent.  Prints one JSON object (integrals/s per workload, the sample
sizes, the machine).  Integrands are the build's built-in families called as
ordinary torch functions (the same expressions the reference would be given).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import platform
import sys
import time
import warnings
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _import_reference(ref_root: str):
    sys.path[:0] = [str(HERE / "refshim"), ref_root, str(REPO)]
    import torchquad  # noqa: F401  (the reference)

    return torchquad


def _cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or "unknown"


def time_c3(tq_ref, budget, dtype):
    """C3 workload (bench.c3_workload): per-call grid rules."""
    import torch

    import bench
    import torchquad_gb300 as tq

    specs, _ = bench.c3_workload()
    cls = {"trapezoid": tq_ref.Trapezoid, "simpson": tq_ref.Simpson, "boole": tq_ref.Boole,
           "gausslegendre": tq_ref.GaussLegendre}
    torch.set_default_dtype(dtype)
    t0 = time.perf_counter()
    k = 0
    while k < len(specs) and time.perf_counter() - t0 < budget:
        rule, d, N, dom, a, u = specs[k]
        f = tq.GaussianPeak(d, a=a.tolist(), u=u.tolist())
        cls[rule]().integrate(f, d, N=N, integration_domain=torch.tensor(dom, dtype=dtype), backend="torch")
        k += 1
    t = time.perf_counter() - t0
    torch.set_default_dtype(torch.float32)
    return {"integrals_per_s": k / t, "sample": f"the first {k} of the 4096 integrals"}


def time_c4(tq_ref, budget):
    """C4's batch of 1024: GL dim 4, 32 nodes, fp64, value and gradients
    (u and the domain bounds require grad), one integral per call."""
    import numpy as np
    import torch

    import torchquad_gb300 as tq

    rng = np.random.default_rng(4)
    a, us = rng.uniform(-3.0, 3.0, (1024, 4)), rng.uniform(0.0, 1.0, 1024)
    t0 = time.perf_counter()
    k = 0
    while k < 1024 and time.perf_counter() - t0 < budget:
        u = torch.tensor(us[k], dtype=torch.float64, requires_grad=True)
        dom = torch.tensor([[0.0, 1.0]] * 4, dtype=torch.float64, requires_grad=True)
        f = tq.Oscillatory(4, a=a[k].tolist(), b=u)
        v = tq_ref.GaussLegendre().integrate(f, 4, N=32**4, integration_domain=dom, backend="torch")
        v.backward()
        k += 1
    t = time.perf_counter() - t0
    return {"integrals_per_s": k / t, "sample": f"the first {k} of the 1024 integrals (forward + backward)"}


def _run_request(tq_ref, r):
    import torch

    dom = torch.tensor(r.domain, dtype=r.dtype)
    if r.method == "montecarlo":
        return tq_ref.MonteCarlo().integrate(r.integrand, r.dim, N=r.N, integration_domain=dom, seed=r.seed,
                                             backend="torch")
    if r.method == "vegas":
        return tq_ref.VEGAS().integrate(r.integrand, r.dim, N=r.N, integration_domain=dom, seed=r.seed,
                                        eps_rel=r.eps_rel, backend="torch")
    return tq_ref.Simpson().integrate(r.integrand, r.dim, N=r.N, integration_domain=dom, backend="torch")


def time_requests(tq_ref, reqs, budget, max_n=None):
    t0 = time.perf_counter()
    k = skipped = 0
    for r in reqs:
        if time.perf_counter() - t0 > budget:
            break
        if max_n is not None and r.N > max_n:
            skipped += 1
            continue
        _run_request(tq_ref, r)
        k += 1
    t = time.perf_counter() - t0
    return k, skipped, t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference")
    ap.add_argument("--budget", type=float, default=20.0)
    args = ap.parse_args()
    tq_ref = _import_reference(args.reference)
    import torch

    import bench

    torch.set_num_threads(os.cpu_count())
    warnings.simplefilter("ignore")
    out = {"machine": {"cpu": _cpu_model(), "threads": torch.get_num_threads(), "torch": torch.__version__},
           "kind": "reference", "budget_s_per_workload": args.budget}
    out["c3_fp64"] = time_c3(tq_ref, args.budget, torch.float64)
    out["c3_fp32"] = time_c3(tq_ref, args.budget, torch.float32)
    out["c4_batch_fwd_bwd"] = time_c4(tq_ref, args.budget)
    reqs = bench.vegas_batch_workload(1024)
    k, _, t = time_requests(tq_ref, reqs, args.budget)
    out["c5_vegas_share"] = {"integrals_per_s": k / t, "sample": f"the first {k} of the 1024 VEGAS requests"}
    from torchquad_gb300.serving import poisson_stream

    stream = [r for _, r in poisson_stream(1000, 1e5, seed=2)]
    k, skipped, t = time_requests(tq_ref, stream, args.budget, max_n=2_000_000)
    out["c5_serving_stream"] = {"integrals_per_s": k / t,
                                "sample": f"{k} requests of the 1000-request stream in arrival order with N <= 2e6 "
                                          f"({skipped} larger ones skipped: minutes each on the CPU)"}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
