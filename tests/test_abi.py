"""The C-ABI library builds, loads and exports every symbol the header
declares (no GPU needed; no compute is called)."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tq_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    import torchquad_gb300.build as B
    from torchquad_gb300 import _lib as L

    B.build()
    handle = L.load(B.lib_path())
    syms = header_symbols()
    assert len(syms) >= 10
    missing = [s for s in syms if not hasattr(handle, s)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert sorted(L.SIGNATURES) == syms


def test_status_strings():
    from torchquad_gb300 import _lib as L

    L.load()
    assert L.status_string(0) == "ok"
    for code in range(-1, -10, -1):
        assert L.status_string(code) != "unknown status"


def test_no_cpu_fallback_without_cuda():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import torchquad_gb300 as tq

    with pytest.raises(RuntimeError, match="no CPU fallback"):
        tq.Simpson().integrate(tq.ExpSum(2), 2, N=9, integration_domain=[[0, 1]] * 2)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        tq.MonteCarlo().integrate(lambda x: x[:, 0], 1, N=10, integration_domain=[[0, 1]])
