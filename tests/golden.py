"""Loaders for the committed golden fixtures (recorded from the unmodified
reference by tests/golden/make_golden.py)."""
import json
from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent / "golden"


@lru_cache(None)
def load(name):
    with open(HERE / name) as fh:
        return json.load(fh)


@lru_cache(None)
def load_npz(name):
    with np.load(HERE / name) as z:
        return {k: z[k] for k in z.files}


def f(h):
    return float.fromhex(h)


def arr(hs):
    return np.array([float.fromhex(h) for h in hs], dtype=np.float64)


RULES = {"Trapezoid": 0, "Simpson": 1, "Boole": 2, "GaussLegendre": 3}
